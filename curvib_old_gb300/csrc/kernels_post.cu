// The steps that follow the flux correction in the reference's Projection
// (poisson.c:2897-2904): Contra2Cart (rhs.c:25-143), the Cartesian velocity at
// the cell centres, and GhostNodeVelocity (bcs.c:3645-4435), its values on the
// boundary ring; Divergence (main.c:469-593), the check after them;
// MetricsDivergence (metrics.c:1551-1625), the set-up check of the metrics;
// and Convection (rhs.c:1463-1946), the convective term of the momentum
// right-hand side.  FP64 with every operation rounded on its own, in the
// reference's order (no fused multiply-add), so results equal the reference's
// bit for bit.  Arrays are the finest level's [mz][my][mx] box, Cmpnts
// interleaved.
#include <functional>

#include "cvb_internal.h"

namespace cvb {

static inline unsigned nblk(size_t n, int t) { return (unsigned)((n + t - 1) / t); }

__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }
__device__ __noinline__ double half_slow(double x) { return dm(0.5, x); }
// 0.5 x, as the FP64 multiply gives it, on the integer pipe: one less in the
// exponent field while the result stays normal, and a zero stays itself.
// Subnormal results, inf and NaN go through the multiply, out of line.
__device__ __forceinline__ double half_exact(double x) {
  const long long b = __double_as_longlong(x), e = (b >> 52) & 0x7ff;
  if (e > 1 && e < 0x7ff) return __longlong_as_double(b - (1LL << 52));
  if ((b & 0x7fffffffffffffffLL) == 0) return x;
  return half_slow(x);
}
__device__ __forceinline__ double mean2(double a, double b) { return half_exact(da(a, b)); }

// Contra2Cart: one thread per interior cell; cells with 0.1 <= nvert <= 7 keep
// their ucat.  The metric rows and fluxes are the means of the cell's two
// faces in each direction.  The metric rows depend on the grid alone, and so
// do the nine 2 x 2 minors of Cramer's rule and the determinant: FAC reads
// them from k_c2c_factors' arrays (the same values, bit for bit) and forms
// only the numerators and the quotients per call.
constexpr int kC2cFactors = 10;  // minors A..I, then the determinant

// The minors b c - d e of the metric rows m, in the order k_contra2cart uses
// them: A = m11 m22 - m12 m21, B = m10 m22 - m12 m20, C = m10 m21 - m11 m20,
// D = m01 m22 - m02 m21, E = m01 m12 - m02 m11, F = m00 m22 - m02 m20,
// G = m00 m12 - m02 m10, H = m00 m21 - m01 m20, I = m00 m11 - m01 m10; and
// det = m00 A - m01 B + m02 C.
__device__ __forceinline__ void c2c_minors(const double (&m)[3][3], double (&f)[kC2cFactors]) {
  auto mn = [](double b, double c, double d, double e) { return ds(dm(b, c), dm(d, e)); };
  f[0] = mn(m[1][1], m[2][2], m[1][2], m[2][1]);
  f[1] = mn(m[1][0], m[2][2], m[1][2], m[2][0]);
  f[2] = mn(m[1][0], m[2][1], m[1][1], m[2][0]);
  f[3] = mn(m[0][1], m[2][2], m[0][2], m[2][1]);
  f[4] = mn(m[0][1], m[1][2], m[0][2], m[1][1]);
  f[5] = mn(m[0][0], m[2][2], m[0][2], m[2][0]);
  f[6] = mn(m[0][0], m[1][2], m[0][2], m[1][0]);
  f[7] = mn(m[0][0], m[2][1], m[0][1], m[2][0]);
  f[8] = mn(m[0][0], m[1][1], m[0][1], m[1][0]);
  f[9] = da(ds(dm(m[0][0], f[0]), dm(m[0][1], f[1])), dm(m[0][2], f[2]));
}

__device__ __forceinline__ void c2c_rows(Geom g, const double *__restrict__ csi, const double *__restrict__ eta,
                                         const double *__restrict__ zet, size_t p, double (&m)[3][3]) {
  const size_t pw = p - 1, ps = p - g.mx, pb = p - (size_t)g.mx * g.my;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    m[0][c] = mean2(csi[3 * pw + c], csi[3 * p + c]);
    m[1][c] = mean2(eta[3 * ps + c], eta[3 * p + c]);
    m[2][c] = mean2(zet[3 * pb + c], zet[3 * p + c]);
  }
}

// The minors and determinant of every interior cell into fac[q N + p].
__global__ void __launch_bounds__(256) k_c2c_factors(Geom g, const double *__restrict__ csi,
                                                     const double *__restrict__ eta, const double *__restrict__ zet,
                                                     double *__restrict__ fac) {
  const int ni = g.mx - 2, nj = g.my - 2;
  const size_t cells = (size_t)ni * nj * (g.mz - 2), n = g.n();
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= cells) return;
  const int i = 1 + (int)(t % ni), j = 1 + (int)((t / ni) % nj), k = 1 + (int)(t / ((size_t)ni * nj));
  const size_t p = ((size_t)k * g.my + j) * g.mx + i;
  double m[3][3], f[kC2cFactors];
  c2c_rows(g, csi, eta, zet, p, m);
  c2c_minors(m, f);
#pragma unroll
  for (int q = 0; q < kC2cFactors; q++) fac[q * n + p] = f[q];
}

template <bool FAC>
__global__ void __launch_bounds__(256) k_contra2cart(Geom g, const double *__restrict__ csi,
                                                     const double *__restrict__ eta, const double *__restrict__ zet,
                                                     const double *__restrict__ fac,
                                                     const double *__restrict__ nvert, const double *__restrict__ uc,
                                                     double *__restrict__ ucat, int k0, int nk) {
  const int ni = g.mx - 2, nj = g.my - 2;
  const size_t cells = (size_t)ni * nj * nk, n = g.n();
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= cells) return;
  const int i = 1 + (int)(t % ni), j = 1 + (int)((t / ni) % nj), k = k0 + (int)(t / ((size_t)ni * nj));
  const size_t p = ((size_t)k * g.my + j) * g.mx + i;
  const double nv = nvert[p];
  if (!(nv < 0.1 || nv > 7.0)) return;
  const size_t pw = p - 1, ps = p - g.mx, pb = p - (size_t)g.mx * g.my;
  double f[kC2cFactors];
  if (FAC) {
#pragma unroll
    for (int q = 0; q < kC2cFactors; q++) f[q] = fac[q * n + p];
  } else {
    double m[3][3];
    c2c_rows(g, csi, eta, zet, p, m);
    c2c_minors(m, f);
  }
  const double q0 = mean2(uc[3 * pw + 0], uc[3 * p + 0]);
  const double q1 = mean2(uc[3 * ps + 1], uc[3 * p + 1]);
  const double q2 = mean2(uc[3 * pb + 2], uc[3 * p + 2]);
  // the numerators of Cramer's rule: q times the minors, in the reference's
  // order (rhs.c:96-118)
  const double d0 = da(ds(dm(q0, f[0]), dm(q1, f[3])), dm(q2, f[4]));
  const double d1 = ds(da(dm(-q0, f[1]), dm(q1, f[5])), dm(q2, f[6]));
  const double d2 = da(ds(dm(q0, f[2]), dm(q1, f[7])), dm(q2, f[8]));
  ucat[3 * p + 0] = __ddiv_rn(d0, f[9]);
  ucat[3 * p + 1] = __ddiv_rn(d1, f[9]);
  ucat[3 * p + 2] = __ddiv_rn(d2, f[9]);
}

// Interior cells of the planes k0 .. k0 + nk - 1 (all interior planes by
// default); fac: k_c2c_factors' arrays, or null to form the minors here.
void launch_contra2cart(const Geom &g, const double *csi, const double *eta, const double *zet,
                        const double *nvert, const double *ucont, double *ucat, cudaStream_t s, int k0, int nk,
                        const double *fac) {
  if (nk < 0) nk = g.mz - 2;
  const size_t cells = (size_t)(g.mx - 2) * (g.my - 2) * nk;
  if (!cells) return;
  if (fac)
    k_contra2cart<true><<<nblk(cells, 256), 256, 0, s>>>(g, csi, eta, zet, fac, nvert, ucont, ucat, k0, nk);
  else
    k_contra2cart<false><<<nblk(cells, 256), 256, 0, s>>>(g, csi, eta, zet, fac, nvert, ucont, ucat, k0, nk);
  count_launch();
}

void launch_c2c_factors(const Geom &g, const double *csi, const double *eta, const double *zet, double *fac,
                        cudaStream_t s) {
  const size_t cells = (size_t)(g.mx - 2) * (g.my - 2) * (g.mz - 2);
  if (!cells) return;
  k_c2c_factors<<<nblk(cells, 256), 256, 0, s>>>(g, csi, eta, zet, fac);
  count_launch();
}

// Divergence (main.c:469-593), the check Flow_Solver runs after Projection:
// |(the cell's three flux differences) * aj| on interior cells, 0 where the
// cell and its face neighbours' nvert sum above 0.1 and on the ring, and the
// maximum with its first index, as VecMax scans for it.  The divergences are
// >= 0, so the pair (largest value, smallest index among equals) is the same
// whatever the reduction order; a NaN never compares greater, as in the scan.
constexpr int kDivThreads = 256, kDivBlocks = 1024;

__device__ __forceinline__ void div_better(double &m, long long &at, double v, long long i) {
  if (v > m || (v == m && i < at)) { m = v; at = i; }
}

__device__ __forceinline__ void div_block_reduce(double m, long long at, double *sv, long long *si) {
  const int t = threadIdx.x;
  sv[t] = m; si[t] = at;
  __syncthreads();
  for (int o = kDivThreads / 2; o > 0; o >>= 1) {
    if (t < o) {
      double a = sv[t];
      long long ai = si[t];
      div_better(a, ai, sv[t + o], si[t + o]);
      sv[t] = a; si[t] = ai;
    }
    __syncthreads();
  }
}

// The quantity of one interior cell p: the flow's divergence (Divergence),
// or with metrics, the divergence of the centre metrics (MetricsDivergence,
// metrics.c:1551-1625), each sum left to right as the C.
__device__ __forceinline__ double flow_div(const Geom &g, const double *uc, const double *aj, const double *nv,
                                          size_t p) {
  const size_t plane = (size_t)g.mx * g.my, w = p - 1, s = p - g.mx, b = p - plane;
  // ((((ux - ux_w) + uy) - uy_s) + uz) - uz_b
  const double sum =
      ds(da(ds(da(ds(uc[3 * p], uc[3 * w]), uc[3 * p + 1]), uc[3 * s + 1]), uc[3 * p + 2]), uc[3 * b + 2]);
  double d = fabs(dm(sum, aj[p]));
  const double ns =
      da(da(da(da(da(da(nv[p], nv[p + plane]), nv[p - plane]), nv[p + g.mx]), nv[p - g.mx]), nv[p + 1]), nv[p - 1]);
  if (ns > 0.1) d = 0.;
  return d;
}
__device__ __forceinline__ double metrics_div(const Geom &g, const double *csi, const double *eta, const double *zet,
                                             const double *aj, size_t p) {
  const size_t w = p - 1, s = p - g.mx, b = p - (size_t)g.mx * g.my;
  double sum = 0.0;
  // csi.x - csi_w.x + eta.x - eta_s.x + zet.x - zet_b.x + (the same for y, z)
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const double t0 = c == 0 ? ds(csi[3 * p], csi[3 * w]) : ds(da(sum, csi[3 * p + c]), csi[3 * w + c]);
    sum = ds(da(ds(da(t0, eta[3 * p + c]), eta[3 * s + c]), zet[3 * p + c]), zet[3 * b + c]);
  }
  return fabs(dm(sum, aj[p]));
}

template <bool METRICS>
__global__ void __launch_bounds__(kDivThreads) k_divergence(Geom g, const double *__restrict__ uc,
                                                          const double *__restrict__ aj,
                                                          const double *__restrict__ nv, const double *__restrict__ csi,
                                                          const double *__restrict__ eta,
                                                          const double *__restrict__ zet, double *pv, long long *pi) {
  __shared__ double sv[kDivThreads];
  __shared__ long long si[kDivThreads];
  double m = -HUGE_VAL;
  long long at = -1;
  const size_t n = g.n(), plane = (size_t)g.mx * g.my;
  for (size_t p = (size_t)blockIdx.x * kDivThreads + threadIdx.x; p < n; p += (size_t)gridDim.x * kDivThreads) {
    const int i = (int)(p % g.mx), j = (int)((p / g.mx) % g.my), k = (int)(p / plane);
    double d = 0.0;
    if (i > 0 && i < g.mx - 1 && j > 0 && j < g.my - 1 && k > 0 && k < g.mz - 1)
      d = METRICS ? metrics_div(g, csi, eta, zet, aj, p) : flow_div(g, uc, aj, nv, p);
    div_better(m, at, d, (long long)p);
  }
  div_block_reduce(m, at, sv, si);
  if (threadIdx.x == 0) { pv[blockIdx.x] = sv[0]; pi[blockIdx.x] = si[0]; }
}

__global__ void __launch_bounds__(kDivThreads) k_divergence_final(const double *pv, const long long *pi, int nb,
                                                                double *out_v, long long *out_i) {
  __shared__ double sv[kDivThreads];
  __shared__ long long si[kDivThreads];
  double m = -HUGE_VAL;
  long long at = -1;
  for (int b = threadIdx.x; b < nb; b += kDivThreads) div_better(m, at, pv[b], pi[b]);
  div_block_reduce(m, at, sv, si);
  if (threadIdx.x == 0) { *out_v = sv[0]; *out_i = si[0]; }
}

void launch_divergence(const Geom &g, const double *ucont, const double *aj, const double *nvert, double *pv,
                       long long *pi, double *out_v, long long *out_i, cudaStream_t s) {
  k_divergence<false><<<kDivBlocks, kDivThreads, 0, s>>>(g, ucont, aj, nvert, nullptr, nullptr, nullptr, pv, pi);
  count_launch();
  k_divergence_final<<<1, kDivThreads, 0, s>>>(pv, pi, kDivBlocks, out_v, out_i);
  count_launch();
}

void launch_metrics_divergence(const Geom &g, const double *csi, const double *eta, const double *zet,
                               const double *aj, double *pv, long long *pi, double *out_v, long long *out_i,
                               cudaStream_t s) {
  k_divergence<true><<<kDivBlocks, kDivThreads, 0, s>>>(g, nullptr, aj, nullptr, csi, eta, zet, pv, pi);
  count_launch();
  k_divergence_final<<<1, kDivThreads, 0, s>>>(pv, pi, kDivBlocks, out_v, out_i);
  count_launch();
}

// ---------------------------------------------------------------- ghost nodes
// A face of the box: f = 2 * axis + side (0: x low, 1: x high, 2: y low, ...).
// Cell (a, b) of face f: for x faces a = j, b = k; for y faces a = i, b = k;
// for z faces a = i, b = j.
struct Face {
  int axis, side;
  __device__ size_t at(const Geom &g, int a, int b, int layer) const {
    // layer: 0 = the ring cell, 1 = its inner neighbour, ... counted from the face
    const int n = axis == 0 ? g.mx : axis == 1 ? g.my : g.mz;
    const int c = side ? n - 1 - layer : layer;
    const int i = axis == 0 ? c : a, j = axis == 1 ? c : (axis == 0 ? a : b), k = axis == 2 ? c : b;
    return ((size_t)k * g.my + j) * g.mx + i;
  }
  __device__ int na(const Geom &g) const { return axis == 0 ? g.my : g.mx; }
  __device__ int nb(const Geom &g) const { return axis == 2 ? g.my : g.mz; }
};

struct GhostArgs {
  Geom g;
  int bc[6];
  const double *csi, *eta, *zet;  // centre metrics
  double *ub, *u;                 // ubcs, ucat
  double *p = nullptr;            // FormBCS: the pressure, averaged on the edges with ucat
  const double *cent = nullptr;   // the cell centres (an annulus face)
  double u_bc = 0.;               // the rheology plates' velocity (bcs.c's U_bc)
};

// The boundary velocity of the special wall types (bcs.c:3776-3975), one face
// per blockIdx.z, the face's interior cells only.  Moving lid (bctype[5] 2)
// and O-grid (bctype[3] 12) faces get a fixed velocity; a slip face (3) the
// tangential part of the velocity next to it, n from the metric of the
// face's outer cell on the low side and of its inner cell on the high side.
// The z-low slip face reads the velocity of its own ring cell, as the
// reference does.
__global__ void k_ghost_special(GhostArgs A) {
  const Geom &g = A.g;
  const int f = blockIdx.z;
  const Face F{f >> 1, f & 1};
  const int a = 1 + blockIdx.x * blockDim.x + threadIdx.x, b = 1 + blockIdx.y * blockDim.y + threadIdx.y;
  if (a > F.na(g) - 2 || b > F.nb(g) - 2) return;
  const size_t p0 = F.at(g, a, b, 0);
  double *ub = A.ub + 3 * p0;
  if (f == 5 && A.bc[5] == 2) { ub[0] = 0.; ub[1] = 1.; ub[2] = 0.; return; }
  if (f == 3 && A.bc[3] == 12) { ub[0] = 0.; ub[1] = 0.; ub[2] = 1.; return; }
  // annulus (bcs.c:3811-3826): (y, -x, 0) / |(x, y)| of the cell centre above
  if (f == 2 && A.bc[2] == 11) {
    const double *c = A.cent + 3 * F.at(g, a, b, 1);
    const double r = __dsqrt_rn(da(dm(c[0], c[0]), dm(c[1], c[1])));
    ub[0] = __ddiv_rn(c[1], r);
    ub[1] = __ddiv_rn(-c[0], r);
    ub[2] = 0.0;
    return;
  }
  // rheology plates (bcs.c:3963-4010): the plate velocity along z on the y
  // faces, along x on the z faces
  if (f >= 2 && A.bc[f] == 13) {
    const double v = (f & 1) ? A.u_bc : -A.u_bc;
    ub[0] = f >= 4 ? v : 0.;
    ub[1] = 0.;
    ub[2] = f >= 4 ? 0. : v;
    return;
  }
  if (A.bc[f] != 3) return;
  const double *met = F.axis == 0 ? A.csi : F.axis == 1 ? A.eta : A.zet;
  const size_t pm = F.side ? F.at(g, a, b, 1) : p0;
  const size_t pu = F.side ? F.at(g, a, b, 1) : (f == 4 ? p0 : F.at(g, a, b, 1));
  const double *m = met + 3 * pm, *u = A.u + 3 * pu;
  const double A2 = __dsqrt_rn(da(da(dm(m[2], m[2]), dm(m[1], m[1])), dm(m[0], m[0])));
  const double nx = __ddiv_rn(m[0], A2), ny = __ddiv_rn(m[1], A2), nz = __ddiv_rn(m[2], A2);
  const double un = da(da(dm(u[0], nx), dm(u[1], ny)), dm(u[2], nz));
  ub[0] = ds(u[0], dm(un, nx));
  ub[1] = ds(u[1], dm(un, ny));
  ub[2] = ds(u[2], dm(un, nz));
}

// Non-periodic ghost faces of one axis, u = 2 ubcs - u(inner neighbour): the
// whole face in GhostNodeVelocity (bcs.c:4015-4076), the face's interior cells
// in FormBCS (interior != 0, bcs.c:5250-5318).
__global__ void k_ghost_faces(GhostArgs A, int axis, int interior) {
  const Geom &g = A.g;
  const Face F{axis, (int)blockIdx.z};
  const int a = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y * blockDim.y + threadIdx.y;
  if (a >= F.na(g) || b >= F.nb(g)) return;
  if (interior && (a < 1 || a > F.na(g) - 2 || b < 1 || b > F.nb(g) - 2)) return;
  const size_t p0 = F.at(g, a, b, 0), p1 = F.at(g, a, b, 1);
#pragma unroll
  for (int c = 0; c < 3; c++) A.u[3 * p0 + c] = ds(dm(2.0, A.ub[3 * p0 + c]), A.u[3 * p1 + c]);
}

// Periodic ring copies of one axis: the ring cell takes the value of the cell
// one period away (cell m-2 for ring cell 0, cell 1 for ring cell m-1).  The
// upper z face copies the x component only, in both rounds, as the reference
// does.  First round (bcs.c:4083-4170): off the face's edges; second round
// (bcs.c:4287-4405): the whole face.
__global__ void k_ghost_ring(GhostArgs A, int axis, int whole) {
  const Geom &g = A.g;
  const Face F{axis, (int)blockIdx.z};
  const int a = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y * blockDim.y + threadIdx.y;
  if (a >= F.na(g) || b >= F.nb(g)) return;
  if (!whole && (a < 1 || a > F.na(g) - 2 || b < 1 || b > F.nb(g) - 2)) return;
  const int n = axis == 0 ? g.mx : axis == 1 ? g.my : g.mz;
  const size_t p0 = F.at(g, a, b, 0), ps = F.at(g, a, b, n - 2);  // ring cell 0 <- m-2, m-1 <- 1
  if (axis == 2 && F.side) {
    A.u[3 * p0] = A.u[3 * ps];
    return;
  }
#pragma unroll
  for (int c = 0; c < 3; c++) A.u[3 * p0 + c] = A.u[3 * ps + c];
}

// The 12 edges of the box (bcs.c:4176-4283; FormBCS's, with p beside ucat,
// bcs.c:5439-5570), each the mean of its two neighbours across the edge, in
// the reference's order: one block, one edge after the other (edges share
// corner cells).
__global__ void k_ghost_edges(GhostArgs A) {
  const Geom &g = A.g;
  const int mx = g.mx, my = g.my, mz = g.mz;
  auto P = [&](int i, int j, int k) { return ((size_t)k * my + j) * mx + i; };
  auto avg = [&](size_t d, size_t a, size_t b) {
#pragma unroll
    for (int c = 0; c < 3; c++) A.u[3 * d + c] = mean2(A.u[3 * a + c], A.u[3 * b + c]);
    if (A.p) A.p[d] = mean2(A.p[a], A.p[b]);
  };
  for (int e = 0; e < 12; e++) {
    const int len = e < 8 ? ((e & 3) < 2 ? my : mx) : mz;
    for (int t = threadIdx.x; t < len; t += blockDim.x) {
      switch (e) {
        case 0: avg(P(0, t, 0), P(0, t, 1), P(1, t, 0)); break;
        case 1: avg(P(mx - 1, t, 0), P(mx - 1, t, 1), P(mx - 2, t, 0)); break;
        case 2: avg(P(t, 0, 0), P(t, 0, 1), P(t, 1, 0)); break;
        case 3: avg(P(t, my - 1, 0), P(t, my - 1, 1), P(t, my - 2, 0)); break;
        case 4: avg(P(0, t, mz - 1), P(0, t, mz - 2), P(1, t, mz - 1)); break;
        case 5: avg(P(mx - 1, t, mz - 1), P(mx - 1, t, mz - 2), P(mx - 2, t, mz - 1)); break;
        case 6: avg(P(t, 0, mz - 1), P(t, 0, mz - 2), P(t, 1, mz - 1)); break;
        case 7: avg(P(t, my - 1, mz - 1), P(t, my - 1, mz - 2), P(t, my - 2, mz - 1)); break;
        case 8: avg(P(0, 0, t), P(0, 1, t), P(1, 0, t)); break;
        case 9: avg(P(mx - 1, 0, t), P(mx - 1, 1, t), P(mx - 2, 0, t)); break;
        case 10: avg(P(0, my - 1, t), P(0, my - 2, t), P(1, my - 1, t)); break;
        default: avg(P(mx - 1, my - 1, t), P(mx - 1, my - 2, t), P(mx - 2, my - 1, t)); break;
      }
    }
    __syncthreads();
  }
}

static void face_grid(const Geom &g, int axis, int faces, dim3 &grd, dim3 &blk) {
  const int na = axis == 0 ? g.my : g.mx, nb = axis == 2 ? g.my : g.mz;
  blk = dim3(32, 8, 1);
  grd = dim3(nblk(na, 32), nblk(nb, 8), faces);
}

void launch_ghost_node_velocity(const Geom &g, const int *bc, const double *csi, const double *eta,
                                const double *zet, double *ubcs, double *ucat, cudaStream_t s, const double *cent,
                                double u_bc) {
  GhostArgs A;
  A.g = g;
  for (int f = 0; f < 6; f++) A.bc[f] = bc[f];
  A.csi = csi; A.eta = eta; A.zet = zet; A.ub = ubcs; A.u = ucat;
  A.cent = cent;
  A.u_bc = u_bc;
  dim3 grd, blk;
  bool special = bc[5] == 2 || bc[3] == 12 || bc[2] == 11;
  for (int f = 0; f < 6; f++) special = special || bc[f] == 3 || (f >= 2 && bc[f] == 13);
  if (special) {
    const int nmax = g.mx > g.my ? (g.mx > g.mz ? g.mx : g.mz) : (g.my > g.mz ? g.my : g.mz);
    k_ghost_special<<<dim3(nblk(nmax, 32), nblk(nmax, 8), 6), dim3(32, 8, 1), 0, s>>>(A);
    count_launch();
  }
  for (int axis = 0; axis < 3; axis++) {
    if (bc[2 * axis] == 7) continue;
    face_grid(g, axis, 2, grd, blk);
    k_ghost_faces<<<grd, blk, 0, s>>>(A, axis, 0);
    count_launch();
  }
  // first round: the three axes touch disjoint cells and read only interior
  // cells, so their order does not matter
  for (int axis = 0; axis < 3; axis++) {
    if (bc[2 * axis] != 7) continue;
    face_grid(g, axis, 2, grd, blk);
    k_ghost_ring<<<grd, blk, 0, s>>>(A, axis, 0);
    count_launch();
  }
  k_ghost_edges<<<1, 256, 0, s>>>(A);
  count_launch();
  for (int axis = 0; axis < 3; axis++) {
    if (bc[2 * axis] != 7) continue;
    face_grid(g, axis, 2, grd, blk);
    k_ghost_ring<<<grd, blk, 0, s>>>(A, axis, 1);
    count_launch();
  }
}

// FormBCS (bcs.c:4436-5889) on a box with walls on its x and y faces and
// walls, or an inlet and an outlet, on its k faces.  Its loop of three passes
// (bcs.c:4483) each runs the outlet's flux correction (outlet_pass, before
// Contra2Cart there), Contra2Cart, the ghost faces on the faces' interior cells
// and the 12 edges of ucat and p.  Contra2Cart reads only ucont, and the faces
// read only interior cells: with walls on the k faces, passes two and three
// give the first pass's values there and only the edges, which read one
// another's cells at the corners, change, so Contra2Cart and the faces run
// once and the edges three times.  With an outlet, a pass changes Ucont.z of
// the last interior k face only, so Contra2Cart runs on that plane alone in
// passes two and three.
void launch_form_bcs(const Geom &g, const double *csi, const double *eta, const double *zet, const double *fac,
                     const double *nvert, double *ucont, double *ubcs, double *ucat, double *p,
                     const std::function<void()> &outlet_pass, cudaStream_t s) {
  GhostArgs A;
  A.g = g;
  for (int f = 0; f < 6; f++) A.bc[f] = 1;
  A.csi = csi; A.eta = eta; A.zet = zet;
  A.ub = ubcs;
  A.u = ucat;
  A.p = p;
  dim3 grd, blk;
  auto faces = [&]() {
    for (int axis = 0; axis < 3; axis++) {
      face_grid(g, axis, 2, grd, blk);
      k_ghost_faces<<<grd, blk, 0, s>>>(A, axis, 1);
      count_launch();
    }
  };
  auto edges = [&]() {
    k_ghost_edges<<<1, 256, 0, s>>>(A);
    count_launch();
  };
  if (!outlet_pass) {
    launch_contra2cart(g, csi, eta, zet, nvert, ucont, ucat, s, 1, -1, fac);
    faces();
    for (int pass = 0; pass < 3; pass++) edges();
    return;
  }
  for (int pass = 0; pass < 3; pass++) {
    outlet_pass();
    if (pass == 0) launch_contra2cart(g, csi, eta, zet, nvert, ucont, ucat, s, 1, -1, fac);
    else launch_contra2cart(g, csi, eta, zet, nvert, ucont, ucat, s, g.mz - 2, 1, fac);
    faces();
    edges();
  }
}

// ---------------------------------------------------------------------------
// Convection (rhs.c:1463-1946).  The face
// fluxes of ucat carried by Ucont/2 are formed once per face by k_conv_faces
// into nine component planes (fp[(3d + c) n + p], coalesced), then
// k_conv_diff takes their differences over each interior cell.  Every product
// and sum is rounded as the C rounds it (no contraction), so the result is the
// reference's bit for bit.  Where the reference reads two cells past the i or
// j end of a row (a face next to the high end whose lower neighbour has nvert
// above 0.1) it reads, on one rank, the first cells of the next row: the flat
// index p + 2 st reads the same, and stays inside the box because the other
// indices are interior.  Along a periodic direction the reference first sets
// the ghost cells just outside the box to the images two cells further out
// (rhs.c:1546-1620) and takes the full QUICK form across the seam where both
// sides are fluid: index -1 reads cell m - 3, index m reads cell 2.

// |x| < 2^1000 (and not NaN), from the exponent field alone
__device__ __forceinline__ bool conv_tame(double x) {
  return (__double_as_longlong(x) & 0x7ff0000000000000LL) < (0x3ffLL + 1000) << 52;
}
__device__ __forceinline__ bool conv_nonzero(double x) { return (__double_as_longlong(x) << 1) != 0; }

// coef * (-x2 - 2 x1 + 3 x0) + x1, the QUICK bracket of either side
__device__ __forceinline__ double conv_bracket(double x2, double x1, double x0) {
  return da(dm(0.125, da(ds(-x2, dm(2., x1)), dm(3., x0))), x1);
}

// 2 x, exactly, for |x| < 2^1000, on the integer pipe: one more in the
// exponent field; a zero or subnormal x doubles its magnitude bits (the IEEE
// encoding runs on from the subnormals into the normals without a seam).
__device__ __forceinline__ double conv_twice(double x) {
  const long long b = __double_as_longlong(x), mag = b & 0x7fffffffffffffffLL;
  return __longlong_as_double((mag >> 52) ? b + (1LL << 52) : (b ^ mag) | (mag << 1));
}
// x / 8 where the result is subnormal: rounded by the FP64 multiply, out of line
__device__ __noinline__ double conv_eighth_tiny(double x) { return dm(0.125, x); }
// 0.125 x, exactly, for finite x: three less in the exponent field while the
// result stays normal; a zero stays itself.
__device__ __forceinline__ double conv_eighth(double x) {
  const long long b = __double_as_longlong(x), e = (b >> 52) & 0x7ff;
  if (e > 3) return __longlong_as_double(b - (3LL << 52));
  if ((b & 0x7fffffffffffffffLL) == 0) return x;
  return conv_eighth_tiny(x);
}
// conv_bracket for inputs below 2^1000, its exact scalings on the integer pipe
__device__ __forceinline__ double conv_bracket_tame(double x2, double x1, double x0) {
  return da(conv_eighth(da(ds(-x2, conv_twice(x1)), dm(3., x0))), x1);
}

// The full face flux um * bracket(u[hi], u[1], u[0]) + up * bracket(u[lo], u[0], u[1]),
// with um = ucon - |ucon|, up = ucon + |ucon|.  Out of line, so that its
// second bracket is evaluated only on this path.
__device__ __noinline__ double conv_quick_full(double ucon, double uh, double u1, double u0, double ul) {
  const double up = da(ucon, fabs(ucon)), um = ds(ucon, fabs(ucon));
  return da(dm(um, conv_bracket(uh, u1, u0)), dm(up, conv_bracket(ul, u0, u1)));
}

// The QUICK face flux of component c.  One of um and up is +0 and the other
// is ucon + ucon.  When ucon and every input are below 2^1000 in magnitude and
// nonzero where it matters, the dead bracket is finite, its product with +0 is
// a zero, and a zero added to the nonzero live product leaves it unchanged: the
// flux is the live product alone, bit for bit, from one bracket on the inputs
// of the upwind side.  A zero live product (whose sign the dead zero could
// change), ucon = 0, NaN or huge values take the full expression.
__device__ __forceinline__ double conv_quick(const double *uc, long long p, long long st, int c, int lo, int hi,
                                            double ucon, bool tame) {
  const double uh = uc[3 * (p + hi * st) + c], u1 = uc[3 * (p + st) + c], u0 = uc[3 * p + c],
               ul = uc[3 * (p + lo * st) + c];
  if (tame && conv_tame(uh) && conv_tame(u1) && conv_tame(u0) && conv_tame(ul)) {
    const bool pos = __double_as_longlong(ucon) >= 0;  // up live (ucon > 0), else um
    const double r = dm(conv_twice(ucon), conv_bracket_tame(pos ? ul : uh, pos ? u0 : u1, pos ? u1 : u0));
    if (conv_nonzero(r)) return r;
  }
  return conv_quick_full(ucon, uh, u1, u0, ul);
}

// n < c and n > c for a positive constant c, as IEEE compares, on the integer
// pipe: a NaN compares false both ways, a negative n (or -0) is below c, and a
// non-negative n orders as its bit pattern does.
__device__ __forceinline__ bool conv_below(double n, double c) {
  const long long b = __double_as_longlong(n), mag = b & 0x7fffffffffffffffLL;
  return mag <= 0x7ff0000000000000LL && (b < 0 || mag < __double_as_longlong(c));
}
__device__ __forceinline__ bool conv_above(double n, double c) {
  const long long b = __double_as_longlong(n);
  return b >= 0 && b <= 0x7ff0000000000000LL && b > __double_as_longlong(c);
}
__device__ __forceinline__ bool conv_fluid(double n) { return conv_below(n, 0.1) || conv_above(n, 7.); }

__global__ void __launch_bounds__(256) k_conv_faces(Geom g, const double *__restrict__ ucont,
                                                   const double *__restrict__ ucat, const double *__restrict__ nv,
                                                   int central, double *__restrict__ fp) {
  const size_t n = g.n(), plane = (size_t)g.mx * g.my;
  for (size_t pu = (size_t)blockIdx.x * blockDim.x + threadIdx.x; pu < n; pu += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(pu % g.mx), j = (int)((pu / g.mx) % g.my), k = (int)(pu / plane);
    const long long p = (long long)pu;
    const int idx[3] = {i, j, k}, ext[3] = {g.mx, g.my, g.mz}, per[3] = {g.px, g.py, g.pz};
    const long long st[3] = {1, g.mx, (long long)plane};
#pragma unroll
    for (int d = 0; d < 3; d++) {
      double f[3] = {0., 0., 0.};
      const int q = idx[d], m = ext[d];
      // the face sweep along d covers q in [0, m-2] with the other two indices interior
      bool on = q <= m - 2;
#pragma unroll
      for (int e = 0; e < 3; e++)
        if (e != d) on = on && idx[e] > 0 && idx[e] < ext[e] - 1;
      if (on) {
        const double ucon = dm(ucont[3 * p + d], 0.5);
        const long long s = st[d];
        // the j sweep tests i (not j) against my-2 for its central end faces
        const bool end2 = d == 1 ? (j == 0 || i == g.my - 2) : (q == 0 || q == m - 2);
        int lo = 0, hi = 0, cen = 0, any = 1;
        if (q > 0 && q < m - 2 && conv_fluid(nv[p + s]) && conv_fluid(nv[p - s])) {
          if (central) cen = 1; else { lo = -1; hi = 2; }
        } else if (central && end2 && conv_fluid(nv[p + s]) && conv_fluid(nv[p])) {
          cen = 1;
        } else if ((d < 2 || q < m - 2) && (q == 0 || conv_above(nv[p - s], 0.1))) {
          // a periodic seam with fluid on both sides takes the full form across
          // it; the reference's ghost cell -1 holds the image of m - 3
          if (per[d] && q == 0 && conv_below(nv[p + (long long)(m - 3) * s], 0.1) && conv_below(nv[p + s], 0.1)) {
            lo = m - 3; hi = 2;
          } else {
            lo = 0; hi = 2;
          }
        } else if ((d < 2 || q > 0) && (q == m - 2 || conv_above(nv[p + s], 0.1))) {
          // ... and its ghost cell m the image of 2
          if (per[d] && q == m - 2 && conv_below(nv[p - s], 0.1) && conv_below(nv[p + s], 0.1)) {
            lo = -1; hi = 4 - m;
          } else {
            lo = -1; hi = 1;
          }
        } else {
          any = 0;
        }
        if (any)
#pragma unroll
          for (int c = 0; c < 3; c++)
            f[c] = cen ? dm(ucon, da(ucat[3 * p + c], ucat[3 * (p + s) + c]))
                       : conv_quick(ucat, p, s, c, lo, hi, ucon, conv_nonzero(ucon) && conv_tame(ucon));
      }
#pragma unroll
      for (int c = 0; c < 3; c++) fp[(size_t)(3 * d + c) * n + pu] = f[c];
    }
  }
}

// conv = fp1 - fp1_w + fp2 - fp2_s + fp3 - fp3_b per component, left to right
// as the C; 0 on the ring.
__global__ void __launch_bounds__(256) k_conv_diff(Geom g, const double *__restrict__ fp, double *__restrict__ conv) {
  const size_t n = g.n(), plane = (size_t)g.mx * g.my;
  for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(p % g.mx), j = (int)((p / g.mx) % g.my), k = (int)(p / plane);
    const bool in = i > 0 && i < g.mx - 1 && j > 0 && j < g.my - 1 && k > 0 && k < g.mz - 1;
#pragma unroll
    for (int c = 0; c < 3; c++) {
      double v = 0.;
      if (in) {
        const double *f1 = fp + (size_t)c * n, *f2 = fp + (size_t)(3 + c) * n, *f3 = fp + (size_t)(6 + c) * n;
        v = ds(da(ds(da(ds(f1[p], f1[p - 1]), f2[p]), f2[p - g.mx]), f3[p]), f3[p - plane]);
      }
      conv[3 * p + c] = v;
    }
  }
}

void launch_convection(const Geom &g, const double *ucont, const double *ucat, const double *nvert, int central,
                       double *fp, double *conv, cudaStream_t s) {
  const size_t n = g.n();
  const unsigned blocks = nblk(n, 256) < 152u * 8 ? nblk(n, 256) : 152u * 8;
  k_conv_faces<<<blocks, 256, 0, s>>>(g, ucont, ucat, nvert, central, fp);
  count_launch();
  k_conv_diff<<<blocks, 256, 0, s>>>(g, fp, conv);
  count_launch();
}

}  // namespace cvb
