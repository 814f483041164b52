// Set-up kernels: face coefficients, switching codes, FP64 stencil weights,
// y-line Thomas factors and the immersed-boundary restriction of nvert.
// Run once per problem (or whenever nvert changes); the solve reuses the result.
#include <algorithm>
#include <vector>

#include "launch.cuh"

namespace cvb {

static inline unsigned nblk(size_t n, int t) { return (unsigned)((n + t - 1) / t); }

// g11..g33 of PoissonLHSNew (poisson.c:699-735): (metric_b . metric_a) * face Jacobian.
__global__ void k_gcoef(Geom g, const double *__restrict__ ic, const double *__restrict__ ie,
                        const double *__restrict__ iz, const double *__restrict__ jc,
                        const double *__restrict__ je, const double *__restrict__ jz,
                        const double *__restrict__ kc, const double *__restrict__ ke,
                        const double *__restrict__ kz, const double *__restrict__ iaj,
                        const double *__restrict__ jaj, const double *__restrict__ kaj,
                        double *__restrict__ g9) {
  size_t n = g.n();
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
    const double *a = ic + 3 * p, *b = ie + 3 * p, *c = iz + 3 * p;
    double j1 = iaj[p];
    g9[0 * n + p] = __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(a[0], a[0]), __dmul_rn(a[1], a[1])), __dmul_rn(a[2], a[2])), j1);
    g9[1 * n + p] = __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(b[0], a[0]), __dmul_rn(b[1], a[1])), __dmul_rn(b[2], a[2])), j1);
    g9[2 * n + p] = __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(c[0], a[0]), __dmul_rn(c[1], a[1])), __dmul_rn(c[2], a[2])), j1);
    a = jc + 3 * p; b = je + 3 * p; c = jz + 3 * p;
    double j2 = jaj[p];
    g9[3 * n + p] = __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(a[0], b[0]), __dmul_rn(a[1], b[1])), __dmul_rn(a[2], b[2])), j2);
    g9[4 * n + p] = __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(b[0], b[0]), __dmul_rn(b[1], b[1])), __dmul_rn(b[2], b[2])), j2);
    g9[5 * n + p] = __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(c[0], b[0]), __dmul_rn(c[1], b[1])), __dmul_rn(c[2], b[2])), j2);
    a = kc + 3 * p; b = ke + 3 * p; c = kz + 3 * p;
    double j3 = kaj[p];
    g9[6 * n + p] = __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(a[0], c[0]), __dmul_rn(a[1], c[1])), __dmul_rn(a[2], c[2])), j3);
    g9[7 * n + p] = __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(b[0], c[0]), __dmul_rn(b[1], c[1])), __dmul_rn(b[2], c[2])), j3);
    g9[8 * n + p] = __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(c[0], c[0]), __dmul_rn(c[1], c[1])), __dmul_rn(c[2], c[2])), j3);
  }
}

void launch_gcoef(const Geom &g, const double *const *m, const double *iaj, const double *jaj,
                  const double *kaj, double *g9, cudaStream_t s) {
  k_gcoef<<<nblk(g.n(), 256), 256, 0, s>>>(g, m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7], m[8],
                                           iaj, jaj, kaj, g9); count_launch();
}

// The cross-derivative form of poisson.c:793-1324: s_up/s_dn are the nvert sums
// of the two cells beside the face one step up/down the cross direction.
__device__ __forceinline__ int cross_branch(double s_up, double s_dn, int c, int m, int per) {
  if ((c == m - 2 && !per) || s_up > 0.1) return (s_dn < 0.1 && (c != 1 || per)) ? 2 : 0;
  if ((c == 1 && !per) || s_dn > 0.1) return (s_up < 0.1) ? 3 : 0;
  return 1;
}

__global__ void k_codes(Geom g, const double *__restrict__ nv, uint32_t *__restrict__ code) {
  size_t n = g.n();
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
    int i = (int)(p % g.mx), j = (int)((p / g.mx) % g.my), k = (int)(p / ((size_t)g.mx * g.my));
    uint32_t c = 0;
    const int mx = g.mx, my = g.my, mz = g.mz;
    auto NV = [&](int a, int b, int d) { return nv[g.id(a, b, d)]; };
    bool inj = j >= 1 && j <= my - 2, ink = k >= 1 && k <= mz - 2, ini = i >= 1 && i <= mx - 2;
    // upper-face cross branches, for every face some interior row can use
    if (inj && ink && i <= mx - 2) {  // E face of (i,j,k)
      c |= (uint32_t)cross_branch(NV(i, j + 1, k) + NV(i + 1, j + 1, k), NV(i, j - 1, k) + NV(i + 1, j - 1, k), j, my, g.py) << 8;
      c |= (uint32_t)cross_branch(NV(i, j, k + 1) + NV(i + 1, j, k + 1), NV(i, j, k - 1) + NV(i + 1, j, k - 1), k, mz, g.pz) << 10;
    }
    if (ini && ink && j <= my - 2) {  // N face
      c |= (uint32_t)cross_branch(NV(i + 1, j, k) + NV(i + 1, j + 1, k), NV(i - 1, j, k) + NV(i - 1, j + 1, k), i, mx, g.px) << 12;
      c |= (uint32_t)cross_branch(NV(i, j, k + 1) + NV(i, j + 1, k + 1), NV(i, j, k - 1) + NV(i, j + 1, k - 1), k, mz, g.pz) << 14;
    }
    if (ini && inj && k <= mz - 2) {  // T face
      c |= (uint32_t)cross_branch(NV(i + 1, j, k) + NV(i + 1, j, k + 1), NV(i - 1, j, k) + NV(i - 1, j, k + 1), i, mx, g.px) << 16;
      c |= (uint32_t)cross_branch(NV(i, j + 1, k) + NV(i, j + 1, k + 1), NV(i, j - 1, k) + NV(i, j - 1, k + 1), j, my, g.py) << 18;
    }
    if (!(ini && inj && ink) || NV(i, j, k) > 0.1) {
      c |= CODE_IDENTITY;
    } else {
      const double thr = 0.1;
      const int x_end = g.px ? mx - 1 : mx - 2, x_str = g.px ? 0 : 1;
      const int y_end = g.py ? my - 1 : my - 2, y_str = g.py ? 0 : 1;
      const int z_end = g.pz ? mz - 1 : mz - 2, z_str = g.pz ? 0 : 1;
      if (NV(i + 1, j, k) < thr && i != x_end) c |= CODE_ACT_E;
      if (NV(i - 1, j, k) < thr && i != x_str) c |= CODE_ACT_W;
      if (NV(i, j + 1, k) < thr && j != y_end) c |= CODE_ACT_N;
      if (NV(i, j - 1, k) < thr && j != y_str) c |= CODE_ACT_S;
      if (NV(i, j, k + 1) < thr && k != z_end) c |= CODE_ACT_T;
      if (NV(i, j, k - 1) < thr && k != z_str) c |= CODE_ACT_B;
    }
    if (NV(i, j, k) > 0.1) c |= CODE_BLOCKED;
    if (ini && inj && ink && NV(i, j, k) < 0.1) c |= CODE_FLUID;
    code[p] = c;
  }
}

__global__ void k_weight32(size_t n, const double *__restrict__ nv, float *__restrict__ w) {
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
    double wt = 1.0 - nv[p];
    w[p] = (float)(wt > 0.0 ? wt : 0.0);
  }
}
void launch_weight32(const Geom &g, const double *nvert, float *wgt32, cudaStream_t s) {
  k_weight32<<<nblk(g.n(), 256) < 4096 ? nblk(g.n(), 256) : 4096, 256, 0, s>>>(g.n(), nvert, wgt32); count_launch();
}

// Any non-zero cross-derivative coefficient (FP32 flux form, after the form
// scaling) or edge weight (FP64 rows) on the level.
__global__ void k_cross_flags(size_t n, const float *__restrict__ gf, const double *__restrict__ w, int *flags) {
  bool f32 = false, f64 = false;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
    f32 |= gf[1 * n + p] != 0.0f || gf[2 * n + p] != 0.0f || gf[3 * n + p] != 0.0f || gf[5 * n + p] != 0.0f ||
           gf[6 * n + p] != 0.0f || gf[7 * n + p] != 0.0f;
    for (int s = NE; s <= BW; s++) f64 |= w[(size_t)s * n + p] != 0.0;
  }
  if (__any_sync(0xffffffffu, f32) && (threadIdx.x & 31) == 0) flags[0] = 1;
  if (__any_sync(0xffffffffu, f64) && (threadIdx.x & 31) == 0) flags[1] = 1;
}
void launch_cross_flags(const Geom &g, const float *gf32, const double *w64, int *flags, cudaStream_t s) {
  k_cross_flags<<<nblk(g.n(), 256) < 4096 ? nblk(g.n(), 256) : 4096, 256, 0, s>>>(g.n(), gf32, w64, flags);
  count_launch();
}

void launch_codes(const Geom &g, const double *nvert, uint32_t *code, cudaStream_t s) {
  k_codes<<<nblk(g.n(), 256), 256, 0, s>>>(g, nvert, code); count_launch();
}

// FP32 flux form: scale each cross-term coefficient by the weight of its form
// (0 none, 1/4 central, 1/2 one-sided), so the apply needs no per-term
// coefficient selection.  Powers of two: the scaling itself is exact.
__global__ void k_scale_cross(Geom g, const uint32_t *__restrict__ code, float *__restrict__ gf) {
  const size_t n = g.n();
  const float wgt[4] = {0.0f, 0.25f, 0.5f, 0.5f};
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
    const uint32_t c = code[p];
    gf[1 * n + p] *= wgt[code_branch(c, 0, 0)];  // g12 (face E, j-direction term)
    gf[2 * n + p] *= wgt[code_branch(c, 0, 1)];  // g13 (face E, k)
    gf[3 * n + p] *= wgt[code_branch(c, 1, 0)];  // g21 (face N, i)
    gf[5 * n + p] *= wgt[code_branch(c, 1, 1)];  // g23 (face N, k)
    gf[6 * n + p] *= wgt[code_branch(c, 2, 0)];  // g31 (face T, i)
    gf[7 * n + p] *= wgt[code_branch(c, 2, 1)];  // g32 (face T, j)
  }
}
void launch_scale_cross(const Geom &g, const uint32_t *code, float *gf32, cudaStream_t s) {
  k_scale_cross<<<nblk(g.n(), 256) < 4096 ? nblk(g.n(), 256) : 4096, 256, 0, s>>>(g, code, gf32); count_launch();
}

// The colour-split copies of a level's 7-point coefficients (row32_split).
__global__ void k_split_coef(Geom g, const float *__restrict__ gf, const float *__restrict__ aj,
                             const uint32_t *__restrict__ code, float *__restrict__ cs) {
  const size_t n = g.n(), S = SplitRow::count(g);
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(p % g.mx), j = (int)((p / g.mx) % g.my), k = (int)(p / ((size_t)g.mx * g.my));
    const size_t q = SplitRow::at(g, i, j, k);
    cs[q] = gf[p];
    cs[S + q] = gf[4 * n + p];
    cs[2 * S + q] = gf[8 * n + p];
    cs[3 * S + q] = aj[p];
    cs[4 * S + q] = __uint_as_float(code[p]);
  }
}
void launch_split_coef(const Geom &g, const float *gf32, const float *ajf32, const uint32_t *code, float *cs,
                       cudaStream_t s) {
  k_split_coef<<<nblk(g.n(), 256) < 4096 ? nblk(g.n(), 256) : 4096, 256, 0, s>>>(g, gf32, ajf32, code, cs);
  count_launch();
}

// One cross term into vol[] in the reference's order (see add_cross in the oracle).
__device__ __forceinline__ void add_cross(double *vol, int br, double gg, bool up, int P, int Q, int Pu,
                                          int Qu, int Pd, int Qd) {
  double h = __dmul_rn(gg, 0.5), q = __dmul_rn(gg, 0.25);
  if (br == 2) {
    if (up) { vol[P] = __dadd_rn(vol[P], h); vol[Q] = __dadd_rn(vol[Q], h); vol[Pd] = __dsub_rn(vol[Pd], h); vol[Qd] = __dsub_rn(vol[Qd], h); }
    else { vol[P] = __dsub_rn(vol[P], h); vol[Q] = __dsub_rn(vol[Q], h); vol[Pd] = __dadd_rn(vol[Pd], h); vol[Qd] = __dadd_rn(vol[Qd], h); }
  } else if (br == 3) {
    if (up) { vol[Pu] = __dadd_rn(vol[Pu], h); vol[Qu] = __dadd_rn(vol[Qu], h); vol[P] = __dsub_rn(vol[P], h); vol[Q] = __dsub_rn(vol[Q], h); }
    else { vol[Pu] = __dsub_rn(vol[Pu], h); vol[Qu] = __dsub_rn(vol[Qu], h); vol[P] = __dadd_rn(vol[P], h); vol[Q] = __dadd_rn(vol[Q], h); }
  } else if (br == 1) {
    if (up) { vol[Pu] = __dadd_rn(vol[Pu], q); vol[Qu] = __dadd_rn(vol[Qu], q); vol[Pd] = __dsub_rn(vol[Pd], q); vol[Qd] = __dsub_rn(vol[Qd], q); }
    else { vol[Pu] = __dsub_rn(vol[Pu], q); vol[Qu] = __dsub_rn(vol[Qu], q); vol[Pd] = __dadd_rn(vol[Pd], q); vol[Qd] = __dadd_rn(vol[Qd], q); }
  }
}

// The 19 matrix entries of one row, accumulated exactly as PoissonLHSNew does
// (poisson.c:789-1327), so the stored weights equal the reference's assembled
// matrix bit for bit.
__global__ void k_weights(Geom g, const double *__restrict__ g9, const double *__restrict__ aj,
                          const uint32_t *__restrict__ code, double *__restrict__ w) {
  size_t n = g.n();
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
    uint32_t c = code[p];
    if (c & CODE_IDENTITY) {
#pragma unroll
      for (int m = 0; m < NSLOT; m++) w[(size_t)m * n + p] = (m == CP) ? 1.0 : 0.0;
      continue;
    }
    int i = (int)(p % g.mx), j = (int)((p / g.mx) % g.my), k = (int)(p / ((size_t)g.mx * g.my));
    double vol[NSLOT];
#pragma unroll
    for (int m = 0; m < NSLOT; m++) vol[m] = 0.0;
    auto G = [&](int q, size_t at) { return g9[(size_t)q * n + at]; };
    size_t pw = g.id(i - 1, j, k), ps = g.id(i, j - 1, k), pb = g.id(i, j, k - 1);
    uint32_t cw = code[pw], cs = code[ps], cb = code[pb];
    if (c & CODE_ACT_E) {
      vol[CP] = __dsub_rn(vol[CP], G(0, p)); vol[EP] = __dadd_rn(vol[EP], G(0, p));
      add_cross(vol, code_branch(c, 0, 0), G(1, p), true, CP, EP, NP, NE, SP, SE);
      add_cross(vol, code_branch(c, 0, 1), G(2, p), true, CP, EP, TP, TE, BP, BE);
    }
    if (c & CODE_ACT_W) {
      vol[CP] = __dsub_rn(vol[CP], G(0, pw)); vol[WP] = __dadd_rn(vol[WP], G(0, pw));
      add_cross(vol, code_branch(cw, 0, 0), G(1, pw), false, CP, WP, NP, NW, SP, SW);
      add_cross(vol, code_branch(cw, 0, 1), G(2, pw), false, CP, WP, TP, TW, BP, BW);
    }
    if (c & CODE_ACT_N) {
      add_cross(vol, code_branch(c, 1, 0), G(3, p), true, CP, NP, EP, NE, WP, NW);
      vol[CP] = __dsub_rn(vol[CP], G(4, p)); vol[NP] = __dadd_rn(vol[NP], G(4, p));
      add_cross(vol, code_branch(c, 1, 1), G(5, p), true, CP, NP, TP, TN, BP, BN);
    }
    if (c & CODE_ACT_S) {
      add_cross(vol, code_branch(cs, 1, 0), G(3, ps), false, CP, SP, EP, SE, WP, SW);
      vol[CP] = __dsub_rn(vol[CP], G(4, ps)); vol[SP] = __dadd_rn(vol[SP], G(4, ps));
      add_cross(vol, code_branch(cs, 1, 1), G(5, ps), false, CP, SP, TP, TS, BP, BS);
    }
    if (c & CODE_ACT_T) {
      add_cross(vol, code_branch(c, 2, 0), G(6, p), true, CP, TP, EP, TE, WP, TW);
      add_cross(vol, code_branch(c, 2, 1), G(7, p), true, CP, TP, NP, TN, SP, TS);
      vol[CP] = __dsub_rn(vol[CP], G(8, p)); vol[TP] = __dadd_rn(vol[TP], G(8, p));
    }
    if (c & CODE_ACT_B) {
      add_cross(vol, code_branch(cb, 2, 0), G(6, pb), false, CP, BP, EP, BE, WP, BW);
      add_cross(vol, code_branch(cb, 2, 1), G(7, pb), false, CP, BP, NP, BN, SP, BS);
      vol[CP] = __dsub_rn(vol[CP], G(8, pb)); vol[BP] = __dadd_rn(vol[BP], G(8, pb));
    }
    double a = -aj[p];
#pragma unroll
    for (int m = 0; m < NSLOT; m++) w[(size_t)m * n + p] = __dmul_rn(vol[m], a);
  }
}

void launch_weights(const Geom &g, const double *g9, const double *aj, const double *nvert,
                    const uint32_t *code, double *w64, cudaStream_t s) {
  (void)nvert;
  k_weights<<<nblk(g.n(), 128), 128, 0, s>>>(g, g9, aj, code, w64); count_launch();
}

// Thomas factors of the in-line (j) part of each row: a_j = w[SP], m_j, c'_j.
// Couplings that wrap around a periodic y seam stay outside the line solve.
__global__ void k_line_factors(Geom g, const double *__restrict__ w, double *__restrict__ l64,
                               float *__restrict__ l32) {
  size_t n = g.n();
  const LineFac F = LineFac::of(g);
  const int Q = F.Q;
  int lines = g.mx * g.mz;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < lines; t += gridDim.x * blockDim.x) {
    int i = t % g.mx, k = t / g.mx;
    const size_t base = F.line(i, k);
    double cprev = 0.0;
    for (int j = 0; j < g.my; j++) {
      size_t p = g.id(i, j, k);
      double a = w[(size_t)SP * n + p], b = w[(size_t)CP * n + p], c = w[(size_t)NP * n + p];
      if (j == 0 || j == g.my - 1) { a = 0.0; c = 0.0; b = 1.0; }
      if (g.py && j == 1) a = 0.0;
      if (g.py && j == g.my - 2) c = 0.0;
      double m = b - a * cprev;
      // an empty row (a fluid cell cut off from all its neighbours) has no
      // pivot: the sweep leaves it unchanged instead of dividing by zero
      double minv = m != 0.0 ? 1.0 / m : 0.0;
      double cp = c * minv;
      if (j >= 1 && j <= g.my - 2) {
        const size_t q = base + (j - 1);
        l64[q] = a; l64[Q + q] = minv; l64[2 * Q + q] = cp;
        l32[q] = (float)a; l32[Q + q] = (float)minv; l32[2 * Q + q] = (float)cp;
      }
      cprev = cp;
    }
    for (int q = g.my - 2; q < Q; q++)  // padding of the runs
      for (int r = 0; r < 3; r++) { l64[base + r * Q + q] = 0.0; l32[base + r * Q + q] = 0.0f; }
  }
}

void launch_line_factors(const Geom &g, const double *w64, double *line64, float *line32,
                         cudaStream_t s) {
  int lines = g.mx * g.mz;
  k_line_factors<<<nblk(lines, 128), 128, 0, s>>>(g, w64, line64, line32); count_launch();
}

__global__ void k_to_f32(const double *__restrict__ a, float *__restrict__ b, size_t n, const int *gate) {
  dep_sync();
  if (gated(gate)) return;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x)
    b[p] = (float)a[p];
}
void launch_to_f32(const double *a, float *b, size_t n, cudaStream_t s, const int *gate) {
  launch_dep(k_to_f32, dim3(nblk(n, 256) < 4096 ? nblk(n, 256) : 4096), 256, 0, s, a, b, n, gate);
}
void launch_f64_to_f32(const double *a, float *b, size_t n, cudaStream_t s, const int *gate) {
  launch_to_f32(a, b, n, s, gate);
}

__global__ void k_to_f64(const float *__restrict__ a, double *__restrict__ b, size_t n, const int *gate) {
  dep_sync();
  if (gated(gate)) return;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x)
    b[p] = (double)a[p];
}
void launch_f32_to_f64(const float *a, double *b, size_t n, cudaStream_t s, const int *gate) {
  launch_dep(k_to_f64, dim3(nblk(n, 256) < 4096 ? nblk(n, 256) : 4096), 256, 0, s, a, b, n, gate);
}

// MyNvertRestriction (poisson.c:1662-1773): a coarse cell is blocked (1) when the
// product of its 8 children's nvert exceeds 0.1; then a fluid coarse cell pinched
// between blocked cells in all three directions is blocked too (second pass reads
// the first pass's result, as the reference's G2L copy does).
__global__ void k_nvert_pass1(Geom F, const double *__restrict__ nf, Geom C, int isc, int jsc, int ksc,
                              double *__restrict__ nc) {
  size_t n = C.n();
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
    int i = (int)(p % C.mx), j = (int)((p / C.mx) % C.my), k = (int)(p / ((size_t)C.mx * C.my));
    double v = 0.0;
    if (i >= 1 && i <= C.mx - 2 && j >= 1 && j <= C.my - 2 && k >= 1 && k <= C.mz - 2) {
      int ih = isc ? i : 2 * i, jh = jsc ? j : 2 * j, kh = ksc ? k : 2 * k;
      int ia = isc ? 0 : 1, ja = jsc ? 0 : 1, ka = ksc ? 0 : 1;
      auto N = [&](int a, int b, int c) { return nf[F.id(a, b, c)]; };
      double prod = N(ih, jh, kh) * N(ih - ia, jh, kh) * N(ih, jh - ja, kh) * N(ih, jh, kh - ka) *
                    N(ih - ia, jh - ja, kh) * N(ih - ia, jh, kh - ka) * N(ih, jh - ja, kh - ka) *
                    N(ih - ia, jh - ja, kh - ka);
      if (prod > 0.1) v = 1.0;
    }
    nc[p] = v;
  }
}
__global__ void k_nvert_pass2(Geom C, const double *__restrict__ snap, double *__restrict__ nc) {
  size_t n = C.n();
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
    int i = (int)(p % C.mx), j = (int)((p / C.mx) % C.my), k = (int)(p / ((size_t)C.mx * C.my));
    if (i >= 1 && i <= C.mx - 2 && j >= 1 && j <= C.my - 2 && k >= 1 && k <= C.mz - 2 && snap[p] < 0.1) {
      if (snap[C.id(i + 1, j, k)] + snap[C.id(i - 1, j, k)] > 1.1 &&
          snap[C.id(i, j + 1, k)] + snap[C.id(i, j - 1, k)] > 1.1 &&
          snap[C.id(i, j, k + 1)] + snap[C.id(i, j, k - 1)] > 1.1)
        nc[p] = 1.0;
    }
  }
}

void launch_nvert_restrict(const Geom &fine, const double *nvf, const Geom &coarse, int isc, int jsc,
                           int ksc, double *nvc, double *tmp, cudaStream_t s) {
  k_nvert_pass1<<<nblk(coarse.n(), 256), 256, 0, s>>>(fine, nvf, coarse, isc, jsc, ksc, tmp); count_launch();
  cudaMemcpyAsync(nvc, tmp, sizeof(double) * coarse.n(), cudaMemcpyDeviceToDevice, s);
  k_nvert_pass2<<<nblk(coarse.n(), 256), 256, 0, s>>>(coarse, tmp, nvc); count_launch();
}

}  // namespace cvb

namespace cvb {

// ------------------------------------------------------------------ dense inverse
// Gauss-Jordan inversion in place with partial pivoting, one column per step,
// for the coarsest level's matrix when it is too large to invert on the host
// in reasonable time (thousands of unknowns).  Step c: k_gj_pivot (one block)
// picks the row of largest |A[r][c]| at or below c (the first of equal ones),
// swaps it into row c, and stages the scaled pivot row (A[c][q] / A[c][c], with
// 1 / A[c][c] in column c, the inverse's column) and the multipliers A[r][c];
// k_gj_elim then updates every row from the staged copies, so no thread reads
// what another writes.  The row swaps become column swaps of the result,
// undone by k_gj_unpermute from the composed column map.
constexpr int kGjThreads = 1024;

__global__ void __launch_bounds__(kGjThreads) k_gj_pivot(double *__restrict__ A, int n, int c, int *__restrict__ perm,
                                                         double *__restrict__ prow, double *__restrict__ fcol,
                                                         int *__restrict__ status) {
  if (*status) return;
  __shared__ double sv[kGjThreads / 32];
  __shared__ int si[kGjThreads / 32];
  __shared__ int s_piv;
  double best = -1.0;
  int bi = n;
  for (int r = c + threadIdx.x; r < n; r += blockDim.x) {
    double v = fabs(A[(size_t)r * n + c]);
    if (v > best) { best = v; bi = r; }  // NaN never wins
  }
  for (int o = 16; o > 0; o >>= 1) {
    double ov = __shfl_down_sync(0xffffffffu, best, o);
    int oi = __shfl_down_sync(0xffffffffu, bi, o);
    if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
  }
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) { sv[wid] = best; si[wid] = bi; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = sv[0];
    int i = si[0];
    for (int w = 1; w < (int)(blockDim.x / 32); w++)
      if (sv[w] > b || (sv[w] == b && si[w] < i)) { b = sv[w]; i = si[w]; }
    if (!(b > 0.0) || i >= n) {
      *status = 1;
      i = -1;
    } else {
      perm[c] = i;
    }
    s_piv = i;
  }
  __syncthreads();
  const int p = s_piv;
  if (p < 0) return;
  if (p != c)
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
      double a = A[(size_t)c * n + q];
      A[(size_t)c * n + q] = A[(size_t)p * n + q];
      A[(size_t)p * n + q] = a;
    }
  __syncthreads();
  const double inv = 1.0 / A[(size_t)c * n + c];
  for (int q = threadIdx.x; q < n; q += blockDim.x)
    prow[q] = q == c ? inv : __dmul_rn(A[(size_t)c * n + q], inv);
  for (int r = threadIdx.x; r < n; r += blockDim.x) fcol[r] = r == c ? 0.0 : A[(size_t)r * n + c];
}

__global__ void k_gj_elim(double *__restrict__ A, int n, int c, const double *__restrict__ prow,
                          const double *__restrict__ fcol, const int *__restrict__ status) {
  if (*status) return;
  const size_t nn = (size_t)n * n;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < nn; e += (size_t)gridDim.x * blockDim.x) {
    int r = (int)(e / n), q = (int)(e % n);
    if (r == c) {
      A[e] = prow[q];
      continue;
    }
    double f = fcol[r];
    if (f == 0.0) continue;  // column c of this row is already 0
    double a = q == c ? 0.0 : A[e];
    A[e] = __dsub_rn(a, __dmul_rn(f, prow[q]));
  }
}

__global__ void k_gj_unpermute(const double *__restrict__ A, int n, const int *__restrict__ colmap,
                               double *__restrict__ out) {
  const size_t nn = (size_t)n * n;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < nn; e += (size_t)gridDim.x * blockDim.x) {
    int r = (int)(e / n), q = (int)(e % n);
    out[e] = A[(size_t)r * n + colmap[q]];
  }
}

// Inverts the n x n row-major A (device, overwritten) into out (device).
// perm / colmap are n ints, prow / fcol n doubles, status one int (device).
// Returns false if a pivot column was all zero (a singular matrix).
bool device_dense_inverse(double *A, int n, double *out, int *perm, int *colmap, double *prow, double *fcol,
                          int *status, cudaStream_t s) {
  cudaMemsetAsync(status, 0, sizeof(int), s);
  const unsigned eb = (unsigned)std::min<size_t>(((size_t)n * n + 255) / 256, (size_t)152 * 16);
  for (int c = 0; c < n; c++) {
    k_gj_pivot<<<1, kGjThreads, 0, s>>>(A, n, c, perm, prow, fcol, status); count_launch();
    k_gj_elim<<<eb, 256, 0, s>>>(A, n, c, prow, fcol, status); count_launch();
  }
  int h_status = 0;
  std::vector<int> h_perm(n), map(n);
  cudaMemcpyAsync(&h_status, status, sizeof(int), cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(h_perm.data(), perm, sizeof(int) * n, cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess || h_status) return false;
  // row swaps (c, perm[c]) in order become column swaps of the inverse in
  // reverse order: out[:, q] = A[:, map[q]]
  for (int q = 0; q < n; q++) map[q] = q;
  for (int c = n - 1; c >= 0; c--) std::swap(map[c], map[h_perm[c]]);
  cudaMemcpyAsync(colmap, map.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s);
  k_gj_unpermute<<<eb, 256, 0, s>>>(A, n, colmap, out); count_launch();
  return cudaStreamSynchronize(s) == cudaSuccess;
}

}  // namespace cvb
