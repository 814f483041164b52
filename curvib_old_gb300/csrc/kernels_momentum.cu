// The momentum right-hand side of the fractional step on the finest level, for
// boxes with no periodic face: Viscous (rhs.c:1947-2566, laminar), FormFunction1
// (rhs.c:2567-3351) and CalcRHS (implicitsolver.c:6449-6713).  FP64, one thread
// per cell.  This file is compiled without multiply-add contraction
// (--fmad=false, build.py), so every product and sum rounds on its own in the
// order the expressions are written -- the reference's C order -- and the
// results equal the reference's bit for bit.
#include "cvb_internal.h"
#include "launch.cuh"

namespace cvb {

namespace {

inline unsigned blocks_for(size_t n, int t) { return (unsigned)((n + t - 1) / t); }

// v > 0.5 && v < 7, on the integer pipe (the kernels here are bound by the
// FP64 one).  As signed 64-bit integers, the bit patterns of doubles of one
// sign compare as the values do; every value with the sign bit (negatives, -0,
// a NaN) lies below 0.5's pattern, and a NaN without it above 7's, so the
// result is the two comparisons', NaN included.
__device__ __forceinline__ bool visc_blocked(double v) {
  const long long b = __double_as_longlong(v);
  return b > 0x3FE0000000000000LL && b < 0x401C000000000000LL;
}

// v > c and v < c for c = 0.1, on the integer pipe.  For c > 0: a pattern
// above c's is a larger positive value, +inf, or a NaN without the sign bit
// (above +inf's pattern), which compares false; a pattern below c's is a
// smaller value of either sign, or a NaN with the sign bit (between -inf's
// pattern and 0 as signed integers), which compares false.
constexpr long long kBits01 = 0x3FB999999999999ALL, kBitsInf = 0x7FF0000000000000LL,
                    kBitsNegInf = (long long)0xFFF0000000000000ULL;
__device__ __forceinline__ bool gt_01(double v) {
  const long long b = __double_as_longlong(v);
  return b > kBits01 && b <= kBitsInf;
}
__device__ __forceinline__ bool lt_01(double v) {
  const long long b = __double_as_longlong(v);
  return b < kBits01 && !(b > kBitsNegInf && b < 0);
}

// x * 2^-K (K = 1, 2) as the FP64 multiply gives it, on the integer pipe while
// the result stays normal: K less in the exponent field; a zero stays itself;
// subnormal results, inf and NaN go through the multiply, out of line.
__device__ __noinline__ double scale_slow(double x, double f) { return x * f; }
template <int K>
__device__ __forceinline__ double scale_down(double x) {
  const long long b = __double_as_longlong(x), e = (b >> 52) & 0x7ff;
  if (e > K && e < 0x7ff) return __longlong_as_double(b - ((long long)K << 52));
  if ((b & 0x7fffffffffffffffLL) == 0) return x;
  return scale_slow(x, K == 1 ? 0.5 : 0.25);
}

struct FaceMetrics {
  const double *m[3][3];  // [face direction][csi, eta, zet] Cmpnts arrays
  const double *aj[3];    // IAj, JAj, KAj
};

}  // namespace

// The viscous flux of every face (rhs.c:2056-2487): face d of cell P, between P
// and P + e_d, into fp[(3 d + c) N + P]; the derivatives across the face's two
// tangential directions are one-sided next to cells with nvert in (0.5, 7).
__global__ void k_visc_faces(Geom g, const double *__restrict__ nv, const double *__restrict__ ucat, FaceMetrics M,
                             const double *__restrict__ gram, double nu, double *__restrict__ fp) {
  const size_t n = g.n();
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % g.mx), j = (int)((e / g.mx) % g.my), k = (int)(e / ((size_t)g.mx * g.my));
    const long P = (long)e;
    const long st[3] = {1, g.mx, (long)g.mx * g.my};
    const int q[3] = {i, j, k}, m[3] = {g.mx, g.my, g.mz};
    for (int d = 0; d < 3; d++) {
      bool in = q[d] <= m[d] - 2;
      for (int t = 0; t < 3; t++)
        if (t != d) in = in && q[t] >= 1 && q[t] <= m[t] - 2;
      if (!in) continue;
      const long sd = st[d];
      double D[3][3];
      for (int c = 0; c < 3; c++) D[d][c] = ucat[3 * (P + sd) + c] - ucat[3 * P + c];
      for (int t = 0; t < 3; t++) {
        if (t == d) continue;
        const long s = st[t];
        const bool up = visc_blocked(nv[P + s]) || visc_blocked(nv[P + sd + s]);
        const bool dn = visc_blocked(nv[P - s]) || visc_blocked(nv[P + sd - s]);
        for (int c = 0; c < 3; c++) {
#define U(off) ucat[3 * (P + (off)) + c]
          if (up) D[t][c] = scale_down<1>(U(sd) + U(0) - U(sd - s) - U(-s));
          else if (dn) D[t][c] = scale_down<1>(U(sd + s) + U(s) - U(sd) - U(0));
          else D[t][c] = scale_down<2>(U(sd + s) + U(s) - U(sd - s) - U(-s));
#undef U
        }
      }
      const double *mc = M.m[d][0] + 3 * P, *me = M.m[d][1] + 3 * P, *mz = M.m[d][2] + 3 * P;
      const double *mm[3] = {mc, me, mz};
      const double *nd = mm[d];
      double gg[3];  // mm[a] . nd, from k_face_gram
      for (int a = 0; a < 3; a++) gg[a] = gram[(size_t)(3 * d + a) * n + e];
      double r[3][3];
      for (int qq = 0; qq < 3; qq++)
        for (int c = 0; c < 3; c++) r[qq][c] = D[0][qq] * mm[0][c] + D[1][qq] * mm[1][c] + D[2][qq] * mm[2][c];
      const double ajc = M.aj[d][P];
      for (int c = 0; c < 3; c++) {
        double v = 0;
        v += (gg[0] * D[0][c] + gg[1] * D[1][c] + gg[2] * D[2][c] + r[0][c] * nd[0] + r[1][c] * nd[1] +
              r[2][c] * nd[2]) * ajc * (nu);
        fp[(size_t)(3 * d + c) * n + e] = v;
      }
    }
  }
}

// visc = the flux differences over each interior cell (rhs.c:2490-2511); 0 on
// the ring (the reference's VecSet before the loops).
__global__ void k_visc_div(Geom g, const double *__restrict__ fp, double *__restrict__ visc) {
  const size_t n = g.n();
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % g.mx), j = (int)((e / g.mx) % g.my), k = (int)(e / ((size_t)g.mx * g.my));
    const bool in = i >= 1 && i <= g.mx - 2 && j >= 1 && j <= g.my - 2 && k >= 1 && k <= g.mz - 2;
    const size_t w = e - 1, s = e - g.mx, b = e - (size_t)g.mx * g.my;
    for (int c = 0; c < 3; c++)
      visc[3 * e + c] = in ? (fp[(size_t)c * n + e] - fp[(size_t)c * n + w] + fp[(size_t)(3 + c) * n + e] -
                              fp[(size_t)(3 + c) * n + s] + fp[(size_t)(6 + c) * n + e] - fp[(size_t)(6 + c) * n + b])
                           : 0.0;
  }
}

// The metric products the viscous flux and FormFunction1's pressure gradient
// both form on every face (rhs.c's g11, g21, g31 of the face): gram[(3 d + a)
// N + P] = M[d][a] . M[d][d] at cell P (x, y, z products summed in that
// order, as the two kernels wrote them).  They depend on the grid alone, so
// they are formed once per grid and read back, the same values bit for bit.
__global__ void k_face_gram(Geom g, FaceMetrics M, double *__restrict__ gram) {
  const size_t n = g.n();
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
    for (int d = 0; d < 3; d++) {
      const double *nd = M.m[d][d] + 3 * e;
      for (int a = 0; a < 3; a++) {
        const double *mm = M.m[d][a] + 3 * e;
        gram[(size_t)(3 * d + a) * n + e] = mm[0] * nd[0] + mm[1] * nd[1] + mm[2] * nd[2];
      }
    }
}

void launch_face_gram(const Geom &g, const double *const *fm, double *gram, cudaStream_t s) {
  FaceMetrics M;
  for (int d = 0; d < 3; d++)
    for (int a = 0; a < 3; a++) M.m[d][a] = fm[3 * d + a];
  k_face_gram<<<blocks_for(g.n(), 256), 256, 0, s>>>(g, M, gram); count_launch();
}

void launch_viscous(const Geom &g, const double *nvert, const double *ucat, const double *const *fm,
                    const double *iaj, const double *jaj, const double *kaj, const double *gram, double nu, double *fp,
                    double *visc, cudaStream_t s) {
  FaceMetrics M;
  for (int d = 0; d < 3; d++)
    for (int a = 0; a < 3; a++) M.m[d][a] = fm[3 * d + a];
  M.aj[0] = iaj; M.aj[1] = jaj; M.aj[2] = kaj;
  const unsigned nb = blocks_for(g.n(), 128);
  k_visc_faces<<<nb, 128, 0, s>>>(g, nvert, ucat, M, gram, nu, fp); count_launch();
  k_visc_div<<<blocks_for(g.n(), 256), 256, 0, s>>>(g, fp, visc); count_launch();
}

// ------------------------------------------------------------- FormFunction1
// rct: the contravariant form of rc = visc - conv at the cell centres
// (rhs.c:2682-2700), interior cells; the ring stays 0 (a new vector).
__global__ void k_ff1_rct(Geom g, const double *__restrict__ conv, const double *__restrict__ visc,
                          const double *__restrict__ csi, const double *__restrict__ eta,
                          const double *__restrict__ zet, const double *__restrict__ aj, double *__restrict__ rct) {
  const size_t n = g.n();
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % g.mx), j = (int)((e / g.mx) % g.my), k = (int)(e / ((size_t)g.mx * g.my));
    if (i < 1 || i > g.mx - 2 || j < 1 || j > g.my - 2 || k < 1 || k > g.mz - 2) {
      rct[3 * e] = rct[3 * e + 1] = rct[3 * e + 2] = 0.0;
      continue;
    }
    const long P = (long)e, sx = 1, sy = g.mx, sz = (long)g.mx * g.my;
    double rc[3];
    for (int c = 0; c < 3; c++) rc[c] = -1.0 * conv[3 * P + c] + visc[3 * P + c];
    const double a = aj[P];
    rct[3 * P + 0] = a * (scale_down<1>(csi[3 * P] + csi[3 * (P - sx)]) * rc[0] +
                          scale_down<1>(csi[3 * P + 1] + csi[3 * (P - sx) + 1]) * rc[1] +
                          scale_down<1>(csi[3 * P + 2] + csi[3 * (P - sx) + 2]) * rc[2]);
    rct[3 * P + 1] = a * (scale_down<1>(eta[3 * P] + eta[3 * (P - sy)]) * rc[0] +
                          scale_down<1>(eta[3 * P + 1] + eta[3 * (P - sy) + 1]) * rc[1] +
                          scale_down<1>(eta[3 * P + 2] + eta[3 * (P - sy) + 2]) * rc[2]);
    rct[3 * P + 2] = a * (scale_down<1>(zet[3 * P] + zet[3 * (P - sz)]) * rc[0] +
                          scale_down<1>(zet[3 * P + 1] + zet[3 * (P - sz) + 1]) * rc[1] +
                          scale_down<1>(zet[3 * P + 2] + zet[3 * (P - sz) + 2]) * rc[2]);
  }
}

namespace {

// One tangential pressure derivative of face d of cell P (rhs.c:2803-2849 and
// its siblings, walled boxes); false where the reference assigns nothing.
__device__ __forceinline__ bool ff_dp(const double *__restrict__ nv, const double *__restrict__ p, long P, long sd,
                                      long s, int q, int m, double &val) {
  const double up = nv[P + s] + nv[P + sd + s], dn = nv[P - s] + nv[P + sd - s];
  if (q == m - 2 || gt_01(up)) {
    if (lt_01(dn) && q != 1) {
      val = scale_down<1>(p[P] + p[P + sd] - p[P - s] - p[P + sd - s]);
      return true;
    }
    return false;
  }
  if (q == 1 || gt_01(dn)) {
    if (lt_01(up)) {
      val = scale_down<1>(p[P + s] + p[P + sd + s] - p[P] - p[P + sd]);
      return true;
    }
    return false;
  }
  val = scale_down<2>(p[P + s] + p[P + sd + s] - p[P - s] - p[P + sd - s]);
  return true;
}

}  // namespace

// The face values of FormFunction1 (rhs.c:2760-3222) and its blocked-face masks
// (rhs.c:3225-3262) on the interior cells.  The reference keeps the three
// derivative variables across its loop: where a branch assigns nothing the
// value of the previous assignment stands.  Within a cell that is the previous
// section's value; entering a cell it is what the previous cell in loop order
// (k, j, i ascending over the interior) left -- its z-section pressure
// derivatives, where its own branch or, failing that, its y-section assigned
// dpde, and its dpdz = p[k+1] - p[k] -- and 0 before the first cell.
__global__ void k_ff1_faces(Geom g, const double *__restrict__ nv, const double *__restrict__ p,
                            const double *__restrict__ rct, FaceMetrics M, const double *__restrict__ gram,
                            double *__restrict__ rhs) {
  const size_t n = g.n();
  const long st[3] = {1, g.mx, (long)g.mx * g.my};
  const int m[3] = {g.mx, g.my, g.mz};
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % g.mx), j = (int)((e / g.mx) % g.my), k = (int)(e / ((size_t)g.mx * g.my));
    if (i < 1 || i > g.mx - 2 || j < 1 || j > g.my - 2 || k < 1 || k > g.mz - 2) continue;
    const long P = (long)e;
    // the previous cell's end values
    double dp[3] = {0.0, 0.0, 0.0};
    {
      int pi = i - 1, pj = j, pk = k;
      if (pi < 1) { pi = g.mx - 2; pj = j - 1; }
      if (pj < 1) { pj = g.my - 2; pk = k - 1; }
      if (pk >= 1) {
        const long Q = ((long)pk * g.my + pj) * g.mx + pi;
        const int qq[3] = {pi, pj, pk};
        // its z section: dpde from the branch, else its y section's p[j+1] - p[j]
        double de;
        if (!ff_dp(nv, p, Q, st[2], st[1], qq[1], m[1], de)) de = p[Q + st[1]] - p[Q];
        dp[1] = de;
        dp[2] = p[Q + st[2]] - p[Q];
        // its final dpdc (the z section's branch, else the y section's, else
        // its x section's p[i+1] - p[i]) is assigned again by this cell's x
        // section before any use
      }
    }
    const int q[3] = {i, j, k};
    double out[3];
    for (int d = 0; d < 3; d++) {
      for (int t = 0; t < 3; t++) {
        if (t == d) dp[t] = p[P + st[d]] - p[P];
        else ff_dp(nv, p, P, st[d], st[t], q[t], m[t], dp[t]);
      }
      // (csi . nd, eta . nd, zet . nd) of face d, from k_face_gram
      const double *gr = gram + (size_t)(3 * d) * n + P;
      double v = scale_down<1>(rct[3 * P + d] + rct[3 * (P + st[d]) + d]);
      v -= (dp[0] * gr[0] + dp[1] * gr[n] + dp[2] * gr[2 * n]) * M.aj[d][P];
      out[d] = v;
    }
    if (gt_01(nv[P])) out[0] = out[1] = out[2] = 0;
    if (gt_01(nv[P + st[0]])) out[0] = 0;
    if (gt_01(nv[P + st[1]])) out[1] = 0;
    if (gt_01(nv[P + st[2]])) out[2] = 0;
    for (int c = 0; c < 3; c++) rhs[3 * P + c] = out[c];
  }
}

void launch_form_function1(const Geom &g, const double *nvert, const double *p, const double *conv,
                           const double *visc, const double *csi, const double *eta, const double *zet,
                           const double *aj, const double *const *fm, const double *iaj, const double *jaj,
                           const double *kaj, const double *gram, double *rct, double *rhs, cudaStream_t s) {
  FaceMetrics M;
  for (int d = 0; d < 3; d++)
    for (int a = 0; a < 3; a++) M.m[d][a] = fm[3 * d + a];
  M.aj[0] = iaj; M.aj[1] = jaj; M.aj[2] = kaj;
  k_ff1_rct<<<blocks_for(g.n(), 256), 256, 0, s>>>(g, conv, visc, csi, eta, zet, aj, rct); count_launch();
  k_ff1_faces<<<blocks_for(g.n(), 128), 128, 0, s>>>(g, nvert, p, rct, M, gram, rhs); count_launch();
}

// ------------------------------------------------------------------ CalcRHS
// After FormFunction1: rhs -= dU / dt over every entry (second-order backward
// dU = 1.5 u - 2 u_o + 0.5 u_rm1, or u - u_o on the first step), the faces
// next to blocked cells and the walls zeroed, the convective-outflow term on
// the last k face (bctype[5] 8), then the reference's six boundary loops,
// which zero the ring except on the box's last row in each direction
// (implicitsolver.c:6519-6713).
__global__ void k_calc_rhs(Geom g, const double *__restrict__ nv, const double *__restrict__ uc,
                           const double *__restrict__ uo, const double *__restrict__ urm, int bdf2, double a,
                           int mz_end, double *__restrict__ rhs) {
  const size_t n = g.n();
  const int mx = g.mx, my = g.my, mz = g.mz;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % mx), j = (int)((e / mx) % my), k = (int)(e / ((size_t)mx * my));
    double r[3];
    for (int c = 0; c < 3; c++) {
      const size_t q = 3 * e + c;
      double du;
      if (bdf2) {
        du = uc[q];
        du *= 1.5;
        du += -2. * uo[q];
        du += scale_down<1>(urm[q]);
      } else {
        du = -1. * uo[q] + uc[q];
      }
      r[c] = rhs[q];
      r[c] += a * du;
    }
    const bool in = i >= 1 && i <= mx - 2 && j >= 1 && j <= my - 2 && k >= 1 && k <= mz - 2;
    if (in) {
      const size_t sx = 1, sy = mx, sz = (size_t)mx * my;
      if (gt_01(nv[e] + nv[e + sx]) || i > mx - 3) r[0] = 0.;
      if (gt_01(nv[e] + nv[e + sy]) || j > my - 3) r[1] = 0.;
      if (gt_01(nv[e] + nv[e + sz]) || k > mz_end) r[2] = 0.;
      if (mz_end == mz - 2 && k == mz - 2) r[2] += 0.8 * (uc[3 * e + 2] - uc[3 * (e - sz) + 2]);
    }
    // the six boundary loops (each covers its face minus the last row of the
    // other two directions)
    const bool kin = k < mz - 1, jin = j < my - 1, iin = i < mx - 1;
    const bool all = ((i == 0 || i == mx - 1) && kin && jin) || ((j == 0 || j == my - 1) && kin && iin) ||
                     ((k == 0 || k == mz - 1) && jin && iin);
    if (all) r[0] = r[1] = r[2] = 0;
    if (i == mx - 2 && kin && jin) r[0] = 0;
    if (j == my - 2 && kin && iin) r[1] = 0;
    if (k == mz - 2 && jin && iin) r[2] = 0;
    for (int c = 0; c < 3; c++) rhs[3 * e + c] = r[c];
  }
}

void launch_calc_rhs(const Geom &g, const double *nvert, const double *ucont, const double *ucont_o,
                     const double *ucont_rm1, int bdf2, double neg_inv_dt, int mz_end, double *rhs, cudaStream_t s) {
  k_calc_rhs<<<blocks_for(g.n(), 256), 256, 0, s>>>(g, nvert, ucont, ucont_o, ucont_rm1, bdf2, neg_inv_dt, mz_end,
                                                     rhs);
  count_launch();
}

// ------------------------------------------------------------------- ImpRK
// One Runge-Kutta stage's update (implicitsolver.c:7156, VecWAXPY):
// u = a rhs + pu over every entry.
__global__ void k_imp_waxpy(size_t n, double a, const double *__restrict__ rhs, const double *__restrict__ pu,
                            double *__restrict__ u) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
    u[e] = a * rhs[e] + pu[e];
}

// The two infinity norms ImpRK takes after its stages (implicitsolver.c:
// 7183-7200): |rhs| and |pu - u| (VecWAXPY(dU, -1, u, pu)), or |rhs| alone
// when pu is null.  The largest |x| is exact in any order; non-negative
// doubles order as their bit patterns, so blocks combine with an integer
// atomicMax into out[0..1] (zeroed by the host).  NaN entries are passed
// over, as a comparison-based maximum passes them.
__global__ void __launch_bounds__(256) k_imp_norms(size_t n, const double *__restrict__ rhs,
                                                   const double *__restrict__ pu, const double *__restrict__ u,
                                                   unsigned long long *out) {
  double mf = 0., md = 0.;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const double f = fabs(rhs[e]);
    if (f > mf) mf = f;
    if (pu) {
      const double d = fabs(-1. * u[e] + pu[e]);
      if (d > md) md = d;
    }
  }
  for (int o = 16; o; o >>= 1) {
    const double f = __shfl_xor_sync(0xffffffffu, mf, o), d = __shfl_xor_sync(0xffffffffu, md, o);
    if (f > mf) mf = f;
    if (d > md) md = d;
  }
  __shared__ double sf[8], sd[8];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) { sf[w] = mf; sd[w] = md; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 1; q < (int)(blockDim.x >> 5); q++) {
      if (sf[q] > mf) mf = sf[q];
      if (sd[q] > md) md = sd[q];
    }
    atomicMax(out, (unsigned long long)__double_as_longlong(mf));
    if (pu) atomicMax(out + 1, (unsigned long long)__double_as_longlong(md));
  }
}

// ------------------------------------------------- InflowFlux, the outlet
// The reference adds a plane's flux and area terms one after another in its
// (j, i) loop.  A chain of dependent FP64 adds is slow on this GPU (one
// thread, about 70 cycles an add: 2.5 ms for a 192 x 192 plane), so the
// kernels below write the terms, in that order, for the host to add; cells
// the reference skips carry +0.0, which leaves a sum that started at +0.0 as
// it was.
//
// The shaped inlet speeds (bcs.c:152-192) at face cell (i, j): the mean of
// its four nodes of the k = 0 node plane (coor0, [my][mx][3]) less the centre
// (cmy, cmz); profile 2 a parabola across y in [0, 4.1] peaking at 1.5, 4 a
// pipe of radius 0.5 peaking at 2, 7 a parabola across y in [-0.5, 0.5]
// peaking at 1.5.  Each product and sum rounded on its own, in the
// reference's order.
__device__ double inlet_shaped(int profile, const double *__restrict__ coor0, int mx, int i, int j, double cmy,
                               double cmz) {
  const double *a = coor0 + 3 * ((size_t)j * mx + i), *b = coor0 + 3 * ((size_t)(j - 1) * mx + i);
  const double *c = coor0 + 3 * ((size_t)j * mx + i - 1), *d = coor0 + 3 * ((size_t)(j - 1) * mx + i - 1);
  const double yc = (a[1] + b[1] + c[1] + d[1]) * 0.25 - cmy;
  const double zc = (a[2] + b[2] + c[2] + d[2]) * 0.25 - cmz;
  const double H = 4.1, Umax = 1.5;
  if (profile == 2) return __ddiv_rn(4. * Umax * yc * (H - yc), H * H);
  if (profile == 4) {
    const double r = __dsqrt_rn(zc * zc + yc * yc);
    return r > 0.5 ? 0. : 2. * (1. - 4. * r * r);
  }
  return 1.5 * (1. - 4. * yc * yc);
}

// InflowFlux on the k = 0 face (bcs.c:148-236): above a fluid cell, ubcs =
// uin zet / |zet| (in the reference's order .y, .z, .x, each its own
// quotient) and Ucont.z = uin |zet|, |zet| summed z, y, x; the face's flux
// terms into terms[(j - 1)(mx - 2) + i - 1].  uin is the constant speed; with
// coor0 set the shaped profile's at the cell, with uin_cell set the speed the
// host formed for the cell (at the terms' index).
__global__ void k_inflow(Geom g, const double *__restrict__ nv, const double *__restrict__ zet, double uin,
                         const double *__restrict__ coor0, int profile, double cmy, double cmz,
                         const double *__restrict__ uin_cell, double *__restrict__ uc, double *__restrict__ ub,
                         double *__restrict__ terms) {
  const int ni = g.mx - 2, n = ni * (g.my - 2);
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = 1 + t % ni, j = 1 + t / ni;
  const size_t q = (size_t)j * g.mx + i;
  double term = 0.;
  if (nv[q + (size_t)g.mx * g.my] < 0.1) {
    if (uin_cell) uin = uin_cell[t];
    else if (coor0) uin = inlet_shaped(profile, coor0, g.mx, i, j, cmy, cmz);
    const double *z = zet + 3 * q;
    const double a = __dsqrt_rn(z[2] * z[2] + z[1] * z[1] + z[0] * z[0]);
    ub[3 * q + 1] = __ddiv_rn(uin * z[1], a);
    ub[3 * q + 2] = __ddiv_rn(uin * z[2], a);
    ub[3 * q + 0] = __ddiv_rn(uin * z[0], a);
    uc[3 * q + 2] = uin * a;
    term = uc[3 * q + 2];
  }
  terms[t] = term;
}

void launch_inflow(const Geom &g, const double *nvert, const double *zet, double uin, const double *coor0,
                   int profile, double cmy, double cmz, const double *uin_cell, double *ucont, double *ubcs,
                   double *terms, cudaStream_t s) {
  const int n = (g.mx - 2) * (g.my - 2);
  k_inflow<<<blocks_for(n, 256), 256, 0, s>>>(g, nvert, zet, uin, coor0, profile, cmy, cmz, uin_cell, ucont, ubcs,
                                              terms);
  count_launch();
}

// The outlet (bcs.c:4914-4940): over the fluid cells of the last interior k
// plane, the flux ucat . zet (x, y, z in order) and the area |zet| (x, y, z)
// into terms[0 .. n) and terms[n .. 2n).
__global__ void k_outlet_terms(Geom g, const double *__restrict__ nv, const double *__restrict__ zet,
                               const double *__restrict__ ucat, double *__restrict__ terms) {
  const int ni = g.mx - 2, n = ni * (g.my - 2);
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = 1 + t % ni, j = 1 + t / ni;
  const size_t q = ((size_t)(g.mz - 2) * g.my + j) * g.mx + i;
  double f = 0., a = 0.;
  if (nv[q] < 0.1) {
    const double *c = ucat + 3 * q, *z = zet + 3 * q;
    f = c[0] * z[0] + c[1] * z[1] + c[2] * z[2];
    a = __dsqrt_rn(z[0] * z[0] + z[1] * z[1] + z[2] * z[2]);
  }
  terms[t] = f;
  terms[n + t] = a;
}

// The outlet's correction (bcs.c:4960-4992) with the ratio the host formed
// from the sums: on the outlet's fluid cells ubcs of the last face = the ucat
// next to it, and Ucont.z of the last interior face = ubcs . zet + ratio
// |zet|.
__global__ void k_outlet_apply(Geom g, const double *__restrict__ nv, const double *__restrict__ zet,
                               const double *__restrict__ ucat, double ratio, double *__restrict__ uc,
                               double *__restrict__ ub) {
  const int ni = g.mx - 2, n = ni * (g.my - 2);
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = 1 + t % ni, j = 1 + t / ni;
  const size_t q = ((size_t)(g.mz - 2) * g.my + j) * g.mx + i, qb = q + (size_t)g.mx * g.my;
  if (!(nv[q] < 0.1)) return;
  const double *c = ucat + 3 * q, *z = zet + 3 * q;
  double b[3];
  for (int k = 0; k < 3; k++) b[k] = ub[3 * qb + k] = c[k];
  uc[3 * q + 2] = (b[0] * z[0] + b[1] * z[1] + b[2] * z[2]) + ratio * __dsqrt_rn(z[0] * z[0] + z[1] * z[1] + z[2] * z[2]);
}

void launch_outlet_terms(const Geom &g, const double *nvert, const double *zet, const double *ucat, double *terms,
                         cudaStream_t s) {
  const int n = (g.mx - 2) * (g.my - 2);
  k_outlet_terms<<<blocks_for(n, 256), 256, 0, s>>>(g, nvert, zet, ucat, terms);
  count_launch();
}

void launch_outlet_apply(const Geom &g, const double *nvert, const double *zet, const double *ucat, double ratio,
                         double *ucont, double *ubcs, cudaStream_t s) {
  const int n = (g.mx - 2) * (g.my - 2);
  k_outlet_apply<<<blocks_for(n, 256), 256, 0, s>>>(g, nvert, zet, ucat, ratio, ucont, ubcs);
  count_launch();
}

void launch_imp_waxpy(size_t n, double a, const double *rhs, const double *pu, double *u, cudaStream_t s) {
  k_imp_waxpy<<<blocks_for(n, 256), 256, 0, s>>>(n, a, rhs, pu, u);
  count_launch();
}

void launch_imp_norms(size_t n, const double *rhs, const double *pu, const double *u, unsigned long long *out,
                      cudaStream_t s) {
  cudaMemsetAsync(out, 0, 2 * sizeof(unsigned long long), s);
  // grid-stride over a few blocks per SM, so that few atomics meet
  const unsigned nb = blocks_for(n, 256) < 2432u ? blocks_for(n, 256) : 2432u;
  k_imp_norms<<<nb, 256, 0, s>>>(n, rhs, pu, u, out);
  count_launch();
}

}  // namespace cvb
