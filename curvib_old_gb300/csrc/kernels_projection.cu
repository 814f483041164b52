// The kernels around the solve: PoissonRHS, VolumeFlux_rev, UpdatePressure and
// the flux correction of Projection.  Element-wise arithmetic keeps the
// reference's operation order (explicit round-to-nearest intrinsics, no fused
// multiply-add); reductions are two-stage and deterministic.
#include "cvb_internal.h"

namespace cvb {

static const int kT = 256;
static inline unsigned nblk(size_t n, int t) { return (unsigned)((n + t - 1) / t); }

__device__ __forceinline__ void block_sum2(double a, double b, double *partial, int nblocks) {
  __shared__ double sh[2][kT / 32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  if (lane == 0) { sh[0][wid] = a; sh[1][wid] = b; }
  __syncthreads();
  if (threadIdx.x < 2) {
    double v = 0.0;
    for (int w = 0; w < kT / 32; w++) v += sh[threadIdx.x][w];
    partial[(size_t)threadIdx.x * nblocks + blockIdx.x] = v;
  }
}

// PoissonRHS (poisson.c:1531-1550) and its compatibility sum (1554-1566).
__global__ void __launch_bounds__(kT) k_rhs(Geom g, const double *__restrict__ uc, const double *__restrict__ aj,
                                            const double *__restrict__ nv, double dt, double st,
                                            double *__restrict__ b, double *partial) {
  double acc = 0.0;
  size_t n = g.n();
  for (size_t p = blockIdx.x * (size_t)kT + threadIdx.x; p < n; p += (size_t)gridDim.x * kT) {
    int i = (int)(p % g.mx), j = (int)((p / g.mx) % g.my), k = (int)(p / ((size_t)g.mx * g.my));
    double v;
    if (i == 0 || i == g.mx - 1 || j == 0 || j == g.my - 1 || k == 0 || k == g.mz - 1 || nv[p] > 0.1) {
      v = 0.0;
    } else {
      double s = __dsub_rn(uc[3 * p], uc[3 * g.id(i - 1, j, k)]);
      s = __dadd_rn(s, uc[3 * p + 1]);
      s = __dsub_rn(s, uc[3 * g.id(i, j - 1, k) + 1]);
      s = __dadd_rn(s, uc[3 * p + 2]);
      s = __dsub_rn(s, uc[3 * g.id(i, j, k - 1) + 2]);
      v = __dmul_rn(__ddiv_rn(__dmul_rn(__ddiv_rn(-s, dt), aj[p]), st), 1.5);
    }
    b[p] = v;
    acc += __ddiv_rn(__dmul_rn(__ddiv_rn(v, aj[p]), dt), 1.5);
  }
  block_sum2(acc, 0.0, partial, gridDim.x);
}
void launch_poisson_rhs(const Geom &g, const double *ucont, const double *aj, const double *nvert, double dt,
                        double st, double *b, double *partial, cudaStream_t s) {
  k_rhs<<<reduce_blocks(), kT, 0, s>>>(g, ucont, aj, nvert, dt, st, b, partial); count_launch();
}

// VolumeFlux_rev sums (poisson.c:3750-3798): flux and face area over the faces
// between fluid (nvert < 0.1) and IB-layer cells (1.1 < nvert < 1.5).
__device__ __forceinline__ bool is_ib(double v) { return v > 1.5 - 0.4 && v < 1.5; }
__global__ void __launch_bounds__(kT) k_ib_sums(Geom g, const double *__restrict__ uc, const double *__restrict__ a3,
                                                const double *__restrict__ nv, double *partial) {
  double f = 0.0, a = 0.0;
  size_t n = g.n();
  for (size_t p = blockIdx.x * (size_t)kT + threadIdx.x; p < n; p += (size_t)gridDim.x * kT) {
    int i = (int)(p % g.mx), j = (int)((p / g.mx) % g.my), k = (int)(p / ((size_t)g.mx * g.my));
    if (i < 1 || i > g.mx - 2 || j < 1 || j > g.my - 2 || k < 1 || k > g.mz - 2) continue;
    double v = nv[p];
    double e = nv[g.id(i + 1, j, k)], nn = nv[g.id(i, j + 1, k)], t = nv[g.id(i, j, k + 1)];
    if (v < 0.1) {
      if (is_ib(e) && i < g.mx - 2) { f += uc[3 * p]; a += a3[p]; }
      if (is_ib(nn) && j < g.my - 2) { f += uc[3 * p + 1]; a += a3[n + p]; }
      if (is_ib(t) && k < g.mz - 2) { f += uc[3 * p + 2]; a += a3[2 * n + p]; }
    }
    if (is_ib(v)) {
      if (e < 0.1 && i < g.mx - 2) { f -= uc[3 * p]; a += a3[p]; }
      if (nn < 0.1 && j < g.my - 2) { f -= uc[3 * p + 1]; a += a3[n + p]; }
      if (t < 0.1 && k < g.mz - 2) { f -= uc[3 * p + 2]; a += a3[2 * n + p]; }
    }
  }
  block_sum2(f, a, partial, gridDim.x);
}
void launch_ib_sums(const Geom &g, const double *ucont, const double *csi, const double *eta, const double *zet,
                    const double *nvert, double *partial, cudaStream_t s) {
  (void)eta; (void)zet;  // csi points at the [3][N] face-area block
  k_ib_sums<<<reduce_blocks(), kT, 0, s>>>(g, ucont, csi, nvert, partial); count_launch();
}

// The uniform correction of VolumeFlux_rev (poisson.c:3810-3869).
__global__ void k_ib_correct(Geom g, double *__restrict__ uc, const double *__restrict__ a3,
                             const double *__restrict__ nv, const double *__restrict__ fa, double fis, int flg) {
  double flux = fa[0], area = fa[1];
  double corr = area > 1.e-15 ? (flg ? __ddiv_rn(__dadd_rn(flux, fis), area) : __ddiv_rn(flux, area)) : 0.0;
  size_t n = g.n();
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
    int i = (int)(p % g.mx), j = (int)((p / g.mx) % g.my), k = (int)(p / ((size_t)g.mx * g.my));
    if (i < 1 || i > g.mx - 2 || j < 1 || j > g.my - 2 || k < 1 || k > g.mz - 2) continue;
    double v = nv[p];
    double e = nv[g.id(i + 1, j, k)], nn = nv[g.id(i, j + 1, k)], t = nv[g.id(i, j, k + 1)];
    if (v < 0.1) {
      if (is_ib(e) && i < g.mx - 2) uc[3 * p] = __dsub_rn(uc[3 * p], __dmul_rn(a3[p], corr));
      if (is_ib(nn) && j < g.my - 2) uc[3 * p + 1] = __dsub_rn(uc[3 * p + 1], __dmul_rn(a3[n + p], corr));
      if (is_ib(t) && k < g.mz - 2) uc[3 * p + 2] = __dsub_rn(uc[3 * p + 2], __dmul_rn(a3[2 * n + p], corr));
    }
    if (is_ib(v)) {
      if (e < 0.1 && i < g.mx - 2) uc[3 * p] = __dadd_rn(uc[3 * p], __dmul_rn(a3[p], corr));
      if (nn < 0.1 && j < g.my - 2) uc[3 * p + 1] = __dadd_rn(uc[3 * p + 1], __dmul_rn(a3[n + p], corr));
      if (t < 0.1 && k < g.mz - 2) uc[3 * p + 2] = __dadd_rn(uc[3 * p + 2], __dmul_rn(a3[2 * n + p], corr));
    }
  }
}
void launch_ib_correct(const Geom &g, double *ucont, const double *csi, const double *eta, const double *zet,
                       const double *nvert, const double *flux_area, double flux_intp_sum, int flg, cudaStream_t s) {
  (void)eta; (void)zet;
  k_ib_correct<<<nblk(g.n(), kT), kT, 0, s>>>(g, ucont, csi, nvert, flux_area, flux_intp_sum, flg); count_launch();
}

// UpdatePressure (poisson.c:2945-3244): p += phi inside, then the periodic ring
// copies, in the reference's order: a first round restricted to interior
// tangential indices (x, y, z), a second round over whole ring planes (x, y, z).
__global__ void k_p_add(Geom g, double *__restrict__ p, const double *__restrict__ phi) {
  size_t n = g.n();
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    int i = (int)(q % g.mx), j = (int)((q / g.mx) % g.my), k = (int)(q / ((size_t)g.mx * g.my));
    if (i >= 1 && i <= g.mx - 2 && j >= 1 && j <= g.my - 2 && k >= 1 && k <= g.mz - 2) p[q] = __dadd_rn(p[q], phi[q]);
  }
}
// axis 0: x ring (plane over j,k); 1: y; 2: z.  restricted: tangential interior only.
__global__ void k_ring_copy(Geom g, double *__restrict__ p, double *__restrict__ phi, int axis, int restricted) {
  int a = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y * blockDim.y + threadIdx.y;
  int na = axis == 0 ? g.my : g.mx, nb = axis == 2 ? g.my : g.mz;
  if (a >= na || b >= nb) return;
  if (restricted) {
    int ma = axis == 0 ? g.my : g.mx, mb = axis == 2 ? g.my : g.mz;
    if (a < 1 || a > ma - 2 || b < 1 || b > mb - 2) return;
  }
  size_t lo, lo_src, hi, hi_src;
  if (axis == 0) { lo = g.id(0, a, b); lo_src = g.id(g.mx - 2, a, b); hi = g.id(g.mx - 1, a, b); hi_src = g.id(1, a, b); }
  else if (axis == 1) { lo = g.id(a, 0, b); lo_src = g.id(a, g.my - 2, b); hi = g.id(a, g.my - 1, b); hi_src = g.id(a, 1, b); }
  else { lo = g.id(a, b, 0); lo_src = g.id(a, b, g.mz - 2); hi = g.id(a, b, g.mz - 1); hi_src = g.id(a, b, 1); }
  p[lo] = p[lo_src]; phi[lo] = phi[lo_src];
  p[hi] = p[hi_src]; phi[hi] = phi[hi_src];
}
void launch_update_pressure(const Geom &g, double *p, double *phi, cudaStream_t s) {
  k_p_add<<<nblk(g.n(), kT), kT, 0, s>>>(g, p, phi); count_launch();
  int per[3] = {g.px, g.py, g.pz};
  if (!(per[0] || per[1] || per[2])) return;
  for (int round = 0; round < 2; round++)
    for (int axis = 0; axis < 3; axis++) {
      if (!per[axis]) continue;
      int na = axis == 0 ? g.my : g.mx, nb = axis == 2 ? g.my : g.mz;
      dim3 blk(32, 8), grd(nblk(na, 32), nblk(nb, 8));
      k_ring_copy<<<grd, blk, 0, s>>>(g, p, phi, axis, round == 0); count_launch();
    }
}

// Projection flux correction (poisson.c:2347-2870).
__device__ __forceinline__ int xbranch(double s_up, double s_dn, int c, int m, int per) {
  if ((c == m - 2 && !per) || s_up > 0.1) return (s_dn < 0.1 && (c != 1 || per)) ? 2 : 0;
  if ((c == 1 && !per) || s_dn > 0.1) return (s_up < 0.1) ? 3 : 0;
  return 1;
}
__device__ __forceinline__ double xdiff(int br, double pu0, double pu1, double p0, double p1, double pd0, double pd1) {
  if (br == 2) return __dmul_rn(__dsub_rn(__dsub_rn(__dadd_rn(p0, p1), pd0), pd1), 0.5);
  if (br == 3) return __dmul_rn(__dsub_rn(__dsub_rn(__dadd_rn(pu0, pu1), p0), p1), 0.5);
  if (br == 1) return __dmul_rn(__dsub_rn(__dsub_rn(__dadd_rn(pu0, pu1), pd0), pd1), 0.25);
  return 0.0;
}
__device__ __forceinline__ double dot3(const double *a, const double *b) {
  return __dadd_rn(__dadd_rn(__dmul_rn(a[0], b[0]), __dmul_rn(a[1], b[1])), __dmul_rn(a[2], b[2]));
}
struct ProjArgs {
  Geom g;
  const double *fm[9];  // ICsi IEta IZet JCsi JEta JZet KCsi KEta KZet (Cmpnts AoS)
  const double *iaj, *jaj, *kaj, *nv, *ph;
  double dt, st;
  double *uc;
};
__device__ __forceinline__ double face_update(const ProjArgs &A, int d, int i, int j, int k) {
  const Geom &g = A.g;
  auto NV = [&](int a, int b, int c) { return A.nv[g.id(a, b, c)]; };
  auto P = [&](int a, int b, int c) { return A.ph[g.id(a, b, c)]; };
  size_t p = g.id(i, j, k);
  double d1, d2, d3, jac;
  const double *m0, *m1, *m2;
  if (d == 0) {
    d1 = __dsub_rn(P(i + 1, j, k), P(i, j, k));
    int bj = xbranch(NV(i, j + 1, k) + NV(i + 1, j + 1, k), NV(i, j - 1, k) + NV(i + 1, j - 1, k), j, g.my, g.py);
    d2 = xdiff(bj, P(i, j + 1, k), P(i + 1, j + 1, k), P(i, j, k), P(i + 1, j, k), P(i, j - 1, k), P(i + 1, j - 1, k));
    int bk = xbranch(NV(i, j, k + 1) + NV(i + 1, j, k + 1), NV(i, j, k - 1) + NV(i + 1, j, k - 1), k, g.mz, g.pz);
    d3 = xdiff(bk, P(i, j, k + 1), P(i + 1, j, k + 1), P(i, j, k), P(i + 1, j, k), P(i, j, k - 1), P(i + 1, j, k - 1));
    m0 = A.fm[0] + 3 * p; m1 = A.fm[1] + 3 * p; m2 = A.fm[2] + 3 * p; jac = A.iaj[p];
    // dpdc*(icsi.icsi)*iaj + dpde*(ieta.icsi)*iaj + dpdz*(izet.icsi)*iaj
    return __dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(d1, dot3(m0, m0)), jac), __dmul_rn(__dmul_rn(d2, dot3(m1, m0)), jac)),
                     __dmul_rn(__dmul_rn(d3, dot3(m2, m0)), jac));
  } else if (d == 1) {
    int bi = xbranch(NV(i + 1, j, k) + NV(i + 1, j + 1, k), NV(i - 1, j, k) + NV(i - 1, j + 1, k), i, g.mx, g.px);
    d1 = xdiff(bi, P(i + 1, j, k), P(i + 1, j + 1, k), P(i, j, k), P(i, j + 1, k), P(i - 1, j, k), P(i - 1, j + 1, k));
    d2 = __dsub_rn(P(i, j + 1, k), P(i, j, k));
    int bk = xbranch(NV(i, j, k + 1) + NV(i, j + 1, k + 1), NV(i, j, k - 1) + NV(i, j + 1, k - 1), k, g.mz, g.pz);
    d3 = xdiff(bk, P(i, j, k + 1), P(i, j + 1, k + 1), P(i, j, k), P(i, j + 1, k), P(i, j, k - 1), P(i, j + 1, k - 1));
    m0 = A.fm[3] + 3 * p; m1 = A.fm[4] + 3 * p; m2 = A.fm[5] + 3 * p; jac = A.jaj[p];
    return __dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(d1, dot3(m0, m1)), jac), __dmul_rn(__dmul_rn(d2, dot3(m1, m1)), jac)),
                     __dmul_rn(__dmul_rn(d3, dot3(m2, m1)), jac));
  } else {
    int bi = xbranch(NV(i + 1, j, k) + NV(i + 1, j, k + 1), NV(i - 1, j, k) + NV(i - 1, j, k + 1), i, g.mx, g.px);
    d1 = xdiff(bi, P(i + 1, j, k), P(i + 1, j, k + 1), P(i, j, k), P(i, j, k + 1), P(i - 1, j, k), P(i - 1, j, k + 1));
    int bj = xbranch(NV(i, j + 1, k) + NV(i, j + 1, k + 1), NV(i, j - 1, k) + NV(i, j - 1, k + 1), j, g.my, g.py);
    d2 = xdiff(bj, P(i, j + 1, k), P(i, j + 1, k + 1), P(i, j, k), P(i, j, k + 1), P(i, j - 1, k), P(i, j - 1, k + 1));
    d3 = __dsub_rn(P(i, j, k + 1), P(i, j, k));
    m0 = A.fm[6] + 3 * p; m1 = A.fm[7] + 3 * p; m2 = A.fm[8] + 3 * p; jac = A.kaj[p];
    return __dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(d1, dot3(m0, m2)), jac), __dmul_rn(__dmul_rn(d2, dot3(m1, m2)), jac)),
                     __dmul_rn(__dmul_rn(d3, dot3(m2, m2)), jac));
  }
}
__device__ __forceinline__ void do_face(const ProjArgs &A, int d, int i, int j, int k) {
  const Geom &g = A.g;
  size_t p = g.id(i, j, k);
  size_t q = d == 0 ? g.id(i + 1, j, k) : (d == 1 ? g.id(i, j + 1, k) : g.id(i, j, k + 1));
  double s = __dadd_rn(A.nv[p], A.nv[q]);
  if (!(s != 0.0)) {
    double f = face_update(A, d, i, j, k);
    A.uc[3 * p + d] = __dsub_rn(A.uc[3 * p + d], __ddiv_rn(__dmul_rn(__dmul_rn(f, A.dt), A.st), 1.5));
  }
}
// Interior faces: each cell updates its own three upper faces (a face belongs to
// exactly one cell, so there is no write conflict).
__global__ void k_projection(ProjArgs A) {
  const Geom &g = A.g;
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
  if (i < 1 || i > g.mx - 2 || j < 1 || j > g.my - 2 || k < 1 || k > g.mz - 2) return;
  int i_end = g.px ? g.mx - 1 : g.mx - 2, j_end = g.py ? g.my - 1 : g.my - 2, k_end = g.pz ? g.mz - 1 : g.mz - 2;
  if (i < i_end) do_face(A, 0, i, j, k);
  if (j < j_end) do_face(A, 1, i, j, k);
  if (k < k_end) do_face(A, 2, i, j, k);
}
// The periodic ring faces (poisson.c:2600-2870): the face between ring cell 0 and cell 1.
__global__ void k_projection_ring(ProjArgs A, int axis) {
  const Geom &g = A.g;
  int a = blockIdx.x * blockDim.x + threadIdx.x + 1, b = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (axis == 0) { if (a > g.my - 2 || b > g.mz - 2) return; do_face(A, 0, 0, a, b); }
  else if (axis == 1) { if (a > g.mx - 2 || b > g.mz - 2) return; do_face(A, 1, a, 0, b); }
  else { if (a > g.mx - 2 || b > g.my - 2) return; do_face(A, 2, a, b, 0); }
}
void launch_projection(const Geom &g, const double *const *fm, const double *iaj, const double *jaj,
                       const double *kaj, const double *nvert, const double *phi, double dt, double st,
                       double *ucont, cudaStream_t s) {
  ProjArgs A;
  A.g = g;
  for (int q = 0; q < 9; q++) A.fm[q] = fm[q];
  A.iaj = iaj; A.jaj = jaj; A.kaj = kaj; A.nv = nvert; A.ph = phi; A.dt = dt; A.st = st; A.uc = ucont;
  dim3 blk(32, 4, 1), grd(nblk(g.mx, 32), nblk(g.my, 4), g.mz);
  k_projection<<<grd, blk, 0, s>>>(A); count_launch();
  int per[3] = {g.px, g.py, g.pz};
  for (int axis = 0; axis < 3; axis++) {
    if (!per[axis]) continue;
    int na = axis == 0 ? g.my : g.mx, nb = axis == 2 ? g.my : g.mz;
    dim3 b2(32, 8), g2(nblk(na, 32), nblk(nb, 8));
    k_projection_ring<<<g2, b2, 0, s>>>(A, axis); count_launch();
  }
}

}  // namespace cvb
