/*
 * TEST INFRASTRUCTURE ONLY: CPU oracle for the pressure-projection path.
 *
 * Each function restates one routine of the reference (CURVIB poisson.c) on
 * plain DMDA-layout arrays, keeping the reference's order of floating-point
 * operations so that results can be compared bit for bit with the reference
 * itself (compiled against the API shim in oracle/petsc_shim/).  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg use this file.
 *
 * Build with -ffp-contract=off: the reference's products are not fused.
 */
#include "cvb_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define COEF 1.5 /* COEF_TIME_ACCURACY, variables.h:421 */

/* stencil slots in the reference's order (poisson.c:576-594) */
enum { CP, EP, WP, NP, SP, TP, BP, NE, SE, NW, SW, TN, BN, TS, BS, TE, BE, TW, BW };

static inline size_t ID(const orc_level *L, int i, int j, int k) {
  return ((size_t)k * L->my + j) * L->mx + i;
}
static inline double NV(const orc_level *L, int i, int j, int k) { return L->nvert[ID(L, i, j, k)]; }
static inline double dot3(const double *a, const double *b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

/* Which one-sided / central form a cross-derivative takes (poisson.c:793-1324
 * and Projection 2347-2870).  s_up / s_dn: nvert sums of the two cells beside
 * the face one step up / down the cross direction; c: the cross index; m: that
 * direction's box size; per: that direction is periodic.
 * 0 none, 1 central (c+1 vs c-1, x0.25), 2 lower (c vs c-1, x0.5),
 * 3 upper (c+1 vs c, x0.5).  The reference's second and fourth branches cannot
 * be reached (each needs the sum its predecessor already rejected). */
static inline int cross_branch(double s_up, double s_dn, int c, int m, int per) {
  if ((c == m - 2 && !per) || s_up > 0.1) {
    if (s_dn < 0.1 && (c != 1 || per)) return 2;
    return 0;
  } else if ((c == 1 && !per) || s_dn > 0.1) {
    if (s_up < 0.1) return 3;
    return 0;
  }
  return 1;
}

/* Face coefficient g_ab of the reference: (metric_b . metric_a) * face Jacobian. */
static inline double gcoef(const double *mb, const double *ma, double jac) {
  return (mb[0] * ma[0] + mb[1] * ma[1] + mb[2] * ma[2]) * jac;
}

/* Add one cross term to vol[].  sign +1 for the upper face (E,N,T) of the row,
 * -1 for the lower face (W,S,B).  P/Q: the row's slot and the face neighbour's
 * slot; Pu,Qu,Pd,Qd: the slots one step up/down the cross direction. */
static inline void add_cross(double *vol, int br, double g, double sign, int P, int Q, int Pu,
                             int Qu, int Pd, int Qd) {
  if (br == 2) {
    if (sign > 0) { vol[P] += g * 0.5; vol[Q] += g * 0.5; vol[Pd] -= g * 0.5; vol[Qd] -= g * 0.5; }
    else { vol[P] -= g * 0.5; vol[Q] -= g * 0.5; vol[Pd] += g * 0.5; vol[Qd] += g * 0.5; }
  } else if (br == 3) {
    if (sign > 0) { vol[Pu] += g * 0.5; vol[Qu] += g * 0.5; vol[P] -= g * 0.5; vol[Q] -= g * 0.5; }
    else { vol[Pu] -= g * 0.5; vol[Qu] -= g * 0.5; vol[P] += g * 0.5; vol[Q] += g * 0.5; }
  } else if (br == 1) {
    if (sign > 0) { vol[Pu] += g * 0.25; vol[Qu] += g * 0.25; vol[Pd] -= g * 0.25; vol[Qd] -= g * 0.25; }
    else { vol[Pu] -= g * 0.25; vol[Qu] -= g * 0.25; vol[Pd] += g * 0.25; vol[Qd] += g * 0.25; }
  }
}

static inline int wrap_up(int i, int m, int per) { return (per && i == m - 2) ? 1 : i + 1; }
static inline int wrap_dn(int i, int m, int per) { return (per && i == 1) ? m - 2 : i - 1; }

int orc_lhs_csr(const orc_level *L, int *rowptr, int *cols, double *vals, int cap) {
  const int mx = L->mx, my = L->my, mz = L->mz;
  const int px = L->bctype[0] == 7, py = L->bctype[2] == 7, pz = L->bctype[4] == 7;
  const int x_end = px ? mx - 1 : mx - 2, x_str = px ? 0 : 1;
  const int y_end = py ? my - 1 : my - 2, y_str = py ? 0 : 1;
  const int z_end = pz ? mz - 1 : mz - 2, z_str = pz ? 0 : 1;
  const double thr = 0.1;
  const size_t N = (size_t)mx * my * mz;
  /* G coefficients over the box (poisson.c:699-735) */
  double *g = (double *)malloc(sizeof(double) * 9 * N);
  for (size_t p = 0; p < N; p++) {
    const double *ic = L->icsi + 3 * p, *ie = L->ieta + 3 * p, *iz = L->izet + 3 * p;
    const double *jc = L->jcsi + 3 * p, *je = L->jeta + 3 * p, *jz = L->jzet + 3 * p;
    const double *kc = L->kcsi + 3 * p, *ke = L->keta + 3 * p, *kz = L->kzet + 3 * p;
    g[9 * p + 0] = gcoef(ic, ic, L->iaj[p]);
    g[9 * p + 1] = gcoef(ie, ic, L->iaj[p]);
    g[9 * p + 2] = gcoef(iz, ic, L->iaj[p]);
    g[9 * p + 3] = gcoef(jc, je, L->jaj[p]);
    g[9 * p + 4] = gcoef(je, je, L->jaj[p]);
    g[9 * p + 5] = gcoef(jz, je, L->jaj[p]);
    g[9 * p + 6] = gcoef(kc, kz, L->kaj[p]);
    g[9 * p + 7] = gcoef(ke, kz, L->kaj[p]);
    g[9 * p + 8] = gcoef(kz, kz, L->kaj[p]);
  }
#define G(n, i, j, k) g[9 * ID(L, i, j, k) + (n)]
  int w = 0;
  rowptr[0] = 0;
  for (int k = 0; k < mz; k++)
    for (int j = 0; j < my; j++)
      for (int i = 0; i < mx; i++) {
        size_t row = ID(L, i, j, k);
        if (i == 0 || i == mx - 1 || j == 0 || j == my - 1 || k == 0 || k == mz - 1 ||
            NV(L, i, j, k) > 0.1) {
          if (w + 1 > cap) { free(g); return -1; }
          cols[w] = (int)row; vals[w] = 1.0; w++;
          rowptr[row + 1] = w;
          continue;
        }
        double vol[19];
        for (int m = 0; m < 19; m++) vol[m] = 0.0;
        double gg;
        /* i+1 - i (poisson.c:794-869) */
        if (NV(L, i + 1, j, k) < thr && i != x_end) {
          vol[CP] -= G(0, i, j, k); vol[EP] += G(0, i, j, k);
          gg = G(1, i, j, k);
          add_cross(vol, cross_branch(NV(L, i, j + 1, k) + NV(L, i + 1, j + 1, k),
                                      NV(L, i, j - 1, k) + NV(L, i + 1, j - 1, k), j, my, py),
                    gg, +1, CP, EP, NP, NE, SP, SE);
          gg = G(2, i, j, k);
          add_cross(vol, cross_branch(NV(L, i, j, k + 1) + NV(L, i + 1, j, k + 1),
                                      NV(L, i, j, k - 1) + NV(L, i + 1, j, k - 1), k, mz, pz),
                    gg, +1, CP, EP, TP, TE, BP, BE);
        }
        /* i - i-1 (poisson.c:872-946) */
        if (NV(L, i - 1, j, k) < thr && i != x_str) {
          vol[CP] -= G(0, i - 1, j, k); vol[WP] += G(0, i - 1, j, k);
          gg = G(1, i - 1, j, k);
          add_cross(vol, cross_branch(NV(L, i, j + 1, k) + NV(L, i - 1, j + 1, k),
                                      NV(L, i, j - 1, k) + NV(L, i - 1, j - 1, k), j, my, py),
                    gg, -1, CP, WP, NP, NW, SP, SW);
          gg = G(2, i - 1, j, k);
          add_cross(vol, cross_branch(NV(L, i, j, k + 1) + NV(L, i - 1, j, k + 1),
                                      NV(L, i, j, k - 1) + NV(L, i - 1, j, k - 1), k, mz, pz),
                    gg, -1, CP, WP, TP, TW, BP, BW);
        }
        /* j+1 - j (poisson.c:949-1056): cross i, main, cross k */
        if (NV(L, i, j + 1, k) < thr && j != y_end) {
          gg = G(3, i, j, k);
          add_cross(vol, cross_branch(NV(L, i + 1, j, k) + NV(L, i + 1, j + 1, k),
                                      NV(L, i - 1, j, k) + NV(L, i - 1, j + 1, k), i, mx, px),
                    gg, +1, CP, NP, EP, NE, WP, NW);
          vol[CP] -= G(4, i, j, k); vol[NP] += G(4, i, j, k);
          gg = G(5, i, j, k);
          add_cross(vol, cross_branch(NV(L, i, j, k + 1) + NV(L, i, j + 1, k + 1),
                                      NV(L, i, j, k - 1) + NV(L, i, j + 1, k - 1), k, mz, pz),
                    gg, +1, CP, NP, TP, TN, BP, BN);
        }
        /* j - j-1 (poisson.c:1059-1165) */
        if (NV(L, i, j - 1, k) < thr && j != y_str) {
          gg = G(3, i, j - 1, k);
          add_cross(vol, cross_branch(NV(L, i + 1, j, k) + NV(L, i + 1, j - 1, k),
                                      NV(L, i - 1, j, k) + NV(L, i - 1, j - 1, k), i, mx, px),
                    gg, -1, CP, SP, EP, SE, WP, SW);
          vol[CP] -= G(4, i, j - 1, k); vol[SP] += G(4, i, j - 1, k);
          gg = G(5, i, j - 1, k);
          add_cross(vol, cross_branch(NV(L, i, j, k + 1) + NV(L, i, j - 1, k + 1),
                                      NV(L, i, j, k - 1) + NV(L, i, j - 1, k - 1), k, mz, pz),
                    gg, -1, CP, SP, TP, TS, BP, BS);
        }
        /* k+1 - k (poisson.c:1168-1245): cross i, cross j, main */
        if (NV(L, i, j, k + 1) < thr && k != z_end) {
          gg = G(6, i, j, k);
          add_cross(vol, cross_branch(NV(L, i + 1, j, k) + NV(L, i + 1, j, k + 1),
                                      NV(L, i - 1, j, k) + NV(L, i - 1, j, k + 1), i, mx, px),
                    gg, +1, CP, TP, EP, TE, WP, TW);
          gg = G(7, i, j, k);
          add_cross(vol, cross_branch(NV(L, i, j + 1, k) + NV(L, i, j + 1, k + 1),
                                      NV(L, i, j - 1, k) + NV(L, i, j - 1, k + 1), j, my, py),
                    gg, +1, CP, TP, NP, TN, SP, TS);
          vol[CP] -= G(8, i, j, k); vol[TP] += G(8, i, j, k);
        }
        /* k - k-1 (poisson.c:1248-1324) */
        if (NV(L, i, j, k - 1) < thr && k != z_str) {
          gg = G(6, i, j, k - 1);
          add_cross(vol, cross_branch(NV(L, i + 1, j, k) + NV(L, i + 1, j, k - 1),
                                      NV(L, i - 1, j, k) + NV(L, i - 1, j, k - 1), i, mx, px),
                    gg, -1, CP, BP, EP, BE, WP, BW);
          gg = G(7, i, j, k - 1);
          add_cross(vol, cross_branch(NV(L, i, j + 1, k) + NV(L, i, j + 1, k - 1),
                                      NV(L, i, j - 1, k) + NV(L, i, j - 1, k - 1), j, my, py),
                    gg, -1, CP, BP, NP, BN, SP, BS);
          vol[CP] -= G(8, i, j, k - 1); vol[BP] += G(8, i, j, k - 1);
        }
        double a = L->aj[row];
        for (int m = 0; m < 19; m++) vol[m] *= -a;
        /* column indices with the periodic wrap (poisson.c:1329-1450) */
        int iu = wrap_up(i, mx, px), id = wrap_dn(i, mx, px);
        int ju = wrap_up(j, my, py), jd = wrap_dn(j, my, py);
        int ku = wrap_up(k, mz, pz), kd = wrap_dn(k, mz, pz);
        int idx[19];
        idx[CP] = (int)ID(L, i, j, k);
        idx[EP] = (int)ID(L, iu, j, k); idx[WP] = (int)ID(L, id, j, k);
        idx[NP] = (int)ID(L, i, ju, k); idx[SP] = (int)ID(L, i, jd, k);
        idx[TP] = (int)ID(L, i, j, ku); idx[BP] = (int)ID(L, i, j, kd);
        idx[NE] = (int)ID(L, iu, ju, k); idx[SE] = (int)ID(L, iu, jd, k);
        idx[NW] = (int)ID(L, id, ju, k); idx[SW] = (int)ID(L, id, jd, k);
        idx[TN] = (int)ID(L, i, ju, ku); idx[BN] = (int)ID(L, i, ju, kd);
        idx[TS] = (int)ID(L, i, jd, ku); idx[BS] = (int)ID(L, i, jd, kd);
        idx[TE] = (int)ID(L, iu, j, ku); idx[BE] = (int)ID(L, iu, j, kd);
        idx[TW] = (int)ID(L, id, j, ku); idx[BW] = (int)ID(L, id, j, kd);
        /* INSERT_VALUES: a repeated column keeps the last value */
        int start = w;
        for (int m = 0; m < 19; m++) {
          int at = -1;
          for (int q = start; q < w; q++) if (cols[q] == idx[m]) { at = q; break; }
          if (at < 0) {
            if (w + 1 > cap) { free(g); return -1; }
            at = w++;
            cols[at] = idx[m];
          }
          vals[at] = vol[m];
        }
        rowptr[row + 1] = w;
      }
#undef G
  free(g);
  return w;
}

void orc_csr_mult(int n, const int *rowptr, const int *cols, const double *vals,
                  const double *x, double *y) {
  for (int r = 0; r < n; r++) {
    double s = 0.0;
    for (int q = rowptr[r]; q < rowptr[r + 1]; q++) s += vals[q] * x[cols[q]];
    y[r] = s;
  }
}

double orc_poisson_rhs(const orc_level *L, const double *uc, double dt, double st, double *b) {
  const int mx = L->mx, my = L->my, mz = L->mz;
  for (int k = 0; k < mz; k++)
    for (int j = 0; j < my; j++)
      for (int i = 0; i < mx; i++) {
        size_t p = ID(L, i, j, k);
        if (i == 0 || i == mx - 1 || j == 0 || j == my - 1 || k == 0 || k == mz - 1) b[p] = 0.;
        else if (L->nvert[p] > 0.1) b[p] = 0;
        else
          b[p] = -(uc[3 * p] - uc[3 * ID(L, i - 1, j, k)] + uc[3 * p + 1] - uc[3 * ID(L, i, j - 1, k) + 1] +
                   uc[3 * p + 2] - uc[3 * ID(L, i, j, k - 1) + 2]) /
                 dt * L->aj[p] / st * COEF;
      }
  double s = 0.;
  for (int k = 0; k < mz; k++)
    for (int j = 0; j < my; j++)
      for (int i = 0; i < mx; i++) {
        size_t p = ID(L, i, j, k);
        s += b[p] / L->aj[p] * dt / COEF;
      }
  return s;
}

static inline double norm3(const double *v) { return sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }

/* One pass of VolumeFlux_rev's sums (poisson.c:3750-3798). */
static void ib_sums(const orc_level *L, const double *uc, double *flux, double *area) {
  const int mx = L->mx, my = L->my, mz = L->mz;
  const double ibmval = 1.5;
  double f = 0, a = 0;
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        size_t p = ID(L, i, j, k);
        double nv = L->nvert[p];
        if (nv < 0.1) {
          double n1 = NV(L, i + 1, j, k), n2 = NV(L, i, j + 1, k), n3 = NV(L, i, j, k + 1);
          if (n1 > ibmval - 0.4 && n1 < ibmval && i < mx - 2) { f += uc[3 * p]; a += norm3(L->csi + 3 * p); }
          if (n2 > ibmval - 0.4 && n2 < ibmval && j < my - 2) { f += uc[3 * p + 1]; a += norm3(L->eta + 3 * p); }
          if (n3 > ibmval - 0.4 && n3 < ibmval && k < mz - 2) { f += uc[3 * p + 2]; a += norm3(L->zet + 3 * p); }
        }
        if (nv > ibmval - 0.4 && nv < ibmval) {
          if (NV(L, i + 1, j, k) < 0.1 && i < mx - 2) { f -= uc[3 * p]; a += norm3(L->csi + 3 * p); }
          if (NV(L, i, j + 1, k) < 0.1 && j < my - 2) { f -= uc[3 * p + 1]; a += norm3(L->eta + 3 * p); }
          if (NV(L, i, j, k + 1) < 0.1 && k < mz - 2) { f -= uc[3 * p + 2]; a += norm3(L->zet + 3 * p); }
        }
      }
  *flux = f;
  *area = a;
}

void orc_volume_flux_rev(const orc_level *L, double *uc, double flux_intp_sum, int flg,
                         double *flux_out, double *area_out) {
  const int mx = L->mx, my = L->my, mz = L->mz;
  const double ibmval = 1.5;
  double flux, area, corr;
  ib_sums(L, uc, &flux, &area);
  if (area > 1.e-15) corr = flg ? (flux + flux_intp_sum) / area : flux / area;
  else corr = 0;
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        size_t p = ID(L, i, j, k);
        double nv = L->nvert[p];
        if (nv < 0.1) {
          double n1 = NV(L, i + 1, j, k), n2 = NV(L, i, j + 1, k), n3 = NV(L, i, j, k + 1);
          if (n1 > ibmval - 0.4 && n1 < ibmval && i < mx - 2) uc[3 * p] -= norm3(L->csi + 3 * p) * corr;
          if (n2 > ibmval - 0.4 && n2 < ibmval && j < my - 2) uc[3 * p + 1] -= norm3(L->eta + 3 * p) * corr;
          if (n3 > ibmval - 0.4 && n3 < ibmval && k < mz - 2) uc[3 * p + 2] -= norm3(L->zet + 3 * p) * corr;
        }
        if (nv > ibmval - 0.4 && nv < ibmval) {
          if (NV(L, i + 1, j, k) < 0.1 && i < mx - 2) uc[3 * p] += norm3(L->csi + 3 * p) * corr;
          if (NV(L, i, j + 1, k) < 0.1 && j < my - 2) uc[3 * p + 1] += norm3(L->eta + 3 * p) * corr;
          if (NV(L, i, j, k + 1) < 0.1 && k < mz - 2) uc[3 * p + 2] += norm3(L->zet + 3 * p) * corr;
        }
      }
  ib_sums(L, uc, flux_out, area_out);
}

void orc_nvert_restrict(const orc_level *F, int cmx, int cmy, int cmz, int coarse_is_level0,
                        int isc, int jsc, int ksc, double *nc) {
  (void)coarse_is_level0; /* both branches of the reference are identical */
  const int ia = isc ? 0 : 1, ja = jsc ? 0 : 1, ka = ksc ? 0 : 1;
  size_t Nc = (size_t)cmx * cmy * cmz;
  for (size_t p = 0; p < Nc; p++) nc[p] = 0.;
#define CI(i, j, k) (((size_t)(k) * cmy + (j)) * cmx + (i))
  for (int k = 1; k < cmz - 1; k++)
    for (int j = 1; j < cmy - 1; j++)
      for (int i = 1; i < cmx - 1; i++) {
        int ih = isc ? i : 2 * i, jh = jsc ? j : 2 * j, kh = ksc ? k : 2 * k;
        if (NV(F, ih, jh, kh) * NV(F, ih - ia, jh, kh) * NV(F, ih, jh - ja, kh) * NV(F, ih, jh, kh - ka) *
                NV(F, ih - ia, jh - ja, kh) * NV(F, ih - ia, jh, kh - ka) * NV(F, ih, jh - ja, kh - ka) *
                NV(F, ih - ia, jh - ja, kh - ka) >
            0.1) {
          double v = nc[CI(i, j, k)];
          nc[CI(i, j, k)] = (1. < v) ? v : 1.;
        }
      }
  /* second pass reads a snapshot (the reference's lNvert after G2L) */
  double *snap = (double *)malloc(sizeof(double) * Nc);
  memcpy(snap, nc, sizeof(double) * Nc);
  for (int k = 1; k < cmz - 1; k++)
    for (int j = 1; j < cmy - 1; j++)
      for (int i = 1; i < cmx - 1; i++) {
        if (nc[CI(i, j, k)] < 0.1) {
          if (snap[CI(i + 1, j, k)] + snap[CI(i - 1, j, k)] > 1.1 &&
              snap[CI(i, j + 1, k)] + snap[CI(i, j - 1, k)] > 1.1 &&
              snap[CI(i, j, k + 1)] + snap[CI(i, j, k - 1)] > 1.1)
            nc[CI(i, j, k)] = 1.;
        }
      }
#undef CI
  free(snap);
}

int orc_fully_blocked(const orc_level *L, int *kske) {
  const int mx = L->mx, my = L->my, mz = L->mz;
  int all = 1;
  memset(kske, 0, sizeof(int) * 2 * (size_t)mx * my);
  for (int j = 1; j < my - 1; j++)
    for (int i = 1; i < mx - 1; i++) {
      int blocked = 0;
      for (int k = 0; k < mz; k++)
        if (NV(L, i, j, k) > 0.1) {
          if (!blocked) { kske[2 * (j * mx + i)] = k; blocked = 1; }
          else if (k < kske[2 * (j * mx + i)]) kske[2 * (j * mx + i)] = k;
        }
      if (!blocked) all = 0;
    }
  return all;
}

void orc_restrict(const orc_level *F, const orc_level *C, const double *x, double *f) {
  const int mx = C->mx, my = C->my, mz = C->mz;
  const int ia = C->isc ? 0 : 1, ja = C->jsc ? 0 : 1, ka = C->ksc ? 0 : 1;
#define W(i, j, k) (x[ID(F, i, j, k)] * ((0. < 1 - NV(F, i, j, k)) ? (1 - NV(F, i, j, k)) : 0.))
  for (int k = 0; k < mz; k++)
    for (int j = 0; j < my; j++)
      for (int i = 0; i < mx; i++) {
        size_t p = ID(C, i, j, k);
        if (k == 0 || k == mz - 1 || j == 0 || j == my - 1 || i == 0 || i == mx - 1) { f[p] = 0.; continue; }
        int ih = C->isc ? i : 2 * i, jh = C->jsc ? j : 2 * j, kh = C->ksc ? k : 2 * k;
        f[p] = 0.125 * (W(ih, jh, kh) + W(ih - ia, jh, kh) + W(ih, jh - ja, kh) + W(ih, jh, kh - ka) +
                        W(ih - ia, jh - ja, kh) + W(ih, jh - ja, kh - ka) + W(ih - ia, jh, kh - ka) +
                        W(ih - ia, jh - ja, kh - ka));
        if (C->nvert[p] > 0.1) f[p] = 0.;
      }
#undef W
}

void orc_interpolate(const orc_level *C, const orc_level *F, const double *x, double *f) {
  const int mx = F->mx, my = F->my, mz = F->mz;
#define XC(i, j, k) x[ID(C, i, j, k)]
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        int ic, jc, kc, ia, ja, ka;
        if (F->isc) { ic = i; ia = 0; }
        else { ic = (i + 1) / 2; ia = (i - 2 * ic) == 0 ? 1 : -1; if (i == 1 || i == mx - 2) ia = 0; }
        if (F->jsc) { jc = j; ja = 0; }
        else { jc = (j + 1) / 2; ja = (j - 2 * jc) == 0 ? 1 : -1; if (j == 1 || j == my - 2) ja = 0; }
        if (F->ksc) { kc = k; ka = 0; }
        else { kc = (k + 1) / 2; ka = (k - 2 * kc) == 0 ? 1 : -1; if (k == 1 || k == mz - 2) ka = 0; }
        if (ka == -1 && NV(C, ic, jc, kc - 1) > 0.1) ka = 0;
        else if (ka == 1 && NV(C, ic, jc, kc + 1) > 0.1) ka = 0;
        if (ja == -1 && NV(C, ic, jc - 1, kc) > 0.1) ja = 0;
        else if (ja == 1 && NV(C, ic, jc + 1, kc) > 0.1) ja = 0;
        if (ia == -1 && NV(C, ic - 1, jc, kc) > 0.1) ia = 0;
        else if (ia == 1 && NV(C, ic + 1, jc, kc) > 0.1) ia = 0;
        f[ID(F, i, j, k)] = (XC(ic, jc, kc) * 9 + XC(ic, jc + ja, kc) * 3 + XC(ic + ia, jc, kc) * 3 +
                             XC(ic + ia, jc + ja, kc)) * 3. / 64. +
                            (XC(ic, jc, kc + ka) * 9 + XC(ic, jc + ja, kc + ka) * 3 +
                             XC(ic + ia, jc, kc + ka) * 3 + XC(ic + ia, jc + ja, kc + ka)) / 64.;
      }
#undef XC
  for (int k = 0; k < mz; k++)
    for (int j = 0; j < my; j++)
      for (int i = 0; i < mx; i++) {
        size_t p = ID(F, i, j, k);
        if (i == 0 || i == mx - 1 || j == 0 || j == my - 1 || k == 0 || k == mz - 1) f[p] = 0.;
        if (F->nvert[p] > 0.1) f[p] = 0.;
      }
}

void orc_nullspace(const orc_level *L, int mns, const int *kske, double *x) {
  const int mx = L->mx, my = L->my, mz = L->mz;
  double sum, num;
  if (!mns) {
    sum = 0; num = 0;
    for (int k = 1; k < mz - 1; k++)
      for (int j = 1; j < my - 1; j++)
        for (int i = 1; i < mx - 1; i++)
          if (NV(L, i, j, k) < 0.1) { sum += x[ID(L, i, j, k)]; num++; }
    sum = sum / (-1.0 * num);
    for (int k = 1; k < mz - 1; k++)
      for (int j = 1; j < my - 1; j++)
        for (int i = 1; i < mx - 1; i++)
          if (NV(L, i, j, k) < 0.1) x[ID(L, i, j, k)] += sum;
  } else {
    for (int side = 0; side < 2; side++) {
      sum = 0; num = 0;
      for (int j = 1; j < my - 1; j++)
        for (int i = 1; i < mx - 1; i++)
          for (int k = 1; k < mz - 1; k++) {
            int below = k < kske[2 * (j * mx + i)];
            if ((side == 0 ? below : !below) && NV(L, i, j, k) < 0.1) { sum += x[ID(L, i, j, k)]; num++; }
          }
      sum /= -num;
      for (int j = 1; j < my - 1; j++)
        for (int i = 1; i < mx - 1; i++)
          for (int k = 1; k < mz - 1; k++) {
            int below = k < kske[2 * (j * mx + i)];
            if ((side == 0 ? below : !below) && NV(L, i, j, k) < 0.1) x[ID(L, i, j, k)] += sum;
          }
    }
  }
  for (int k = 0; k < mz; k++)
    for (int j = 0; j < my; j++)
      for (int i = 0; i < mx; i++)
        if (i == 0 || i == mx - 1 || j == 0 || j == my - 1 || k == 0 || k == mz - 1 || NV(L, i, j, k) > 0.1)
          x[ID(L, i, j, k)] = 0.;
}

void orc_update_pressure(const orc_level *L, double *p, double *phi) {
  const int mx = L->mx, my = L->my, mz = L->mz;
  const int IM = mx - 1, JM = my - 1, KM = mz - 1;
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) p[ID(L, i, j, k)] += phi[ID(L, i, j, k)];
  if (!(L->bctype[0] == 7 || L->bctype[2] == 7 || L->bctype[4] == 7)) return;
  /* each pass reads the ghost image refreshed before it: [-2] -> m-2, [m+1] -> 1 */
  if (L->bctype[0] == 7 || L->bctype[1] == 7)
    for (int k = 0; k < mz; k++)
      for (int j = 0; j < my; j++)
        if (k > 0 && k < KM && j > 0 && j < JM) {
          p[ID(L, 0, j, k)] = p[ID(L, mx - 2, j, k)]; phi[ID(L, 0, j, k)] = phi[ID(L, mx - 2, j, k)];
          p[ID(L, mx - 1, j, k)] = p[ID(L, 1, j, k)]; phi[ID(L, mx - 1, j, k)] = phi[ID(L, 1, j, k)];
        }
  if (L->bctype[2] == 7 || L->bctype[3] == 7)
    for (int k = 0; k < mz; k++)
      for (int i = 0; i < mx; i++)
        if (k > 0 && k < KM && i > 0 && i < IM) {
          p[ID(L, i, 0, k)] = p[ID(L, i, my - 2, k)]; phi[ID(L, i, 0, k)] = phi[ID(L, i, my - 2, k)];
          p[ID(L, i, my - 1, k)] = p[ID(L, i, 1, k)]; phi[ID(L, i, my - 1, k)] = phi[ID(L, i, 1, k)];
        }
  if (L->bctype[4] == 7 || L->bctype[5] == 7)
    for (int j = 0; j < my; j++)
      for (int i = 0; i < mx; i++)
        if (i > 0 && i < IM && j > 0 && j < JM) {
          p[ID(L, i, j, 0)] = p[ID(L, i, j, mz - 2)]; phi[ID(L, i, j, 0)] = phi[ID(L, i, j, mz - 2)];
          p[ID(L, i, j, mz - 1)] = p[ID(L, i, j, 1)]; phi[ID(L, i, j, mz - 1)] = phi[ID(L, i, j, 1)];
        }
  /* second round over whole ring planes (poisson.c:3085-3240): x, then y, then z */
  if (L->bctype[0] == 7 || L->bctype[1] == 7)
    for (int k = 0; k < mz; k++)
      for (int j = 0; j < my; j++) {
        p[ID(L, 0, j, k)] = p[ID(L, mx - 2, j, k)]; phi[ID(L, 0, j, k)] = phi[ID(L, mx - 2, j, k)];
        p[ID(L, mx - 1, j, k)] = p[ID(L, 1, j, k)]; phi[ID(L, mx - 1, j, k)] = phi[ID(L, 1, j, k)];
      }
  if (L->bctype[2] == 7 || L->bctype[3] == 7)
    for (int k = 0; k < mz; k++)
      for (int i = 0; i < mx; i++) {
        p[ID(L, i, my - 1, k)] = p[ID(L, i, 1, k)]; phi[ID(L, i, my - 1, k)] = phi[ID(L, i, 1, k)];
        p[ID(L, i, 0, k)] = p[ID(L, i, my - 2, k)]; phi[ID(L, i, 0, k)] = phi[ID(L, i, my - 2, k)];
      }
  if (L->bctype[4] == 7 || L->bctype[5] == 7)
    for (int j = 0; j < my; j++)
      for (int i = 0; i < mx; i++) {
        p[ID(L, i, j, mz - 1)] = p[ID(L, i, j, 1)]; phi[ID(L, i, j, mz - 1)] = phi[ID(L, i, j, 1)];
        p[ID(L, i, j, 0)] = p[ID(L, i, j, mz - 2)]; phi[ID(L, i, j, 0)] = phi[ID(L, i, j, mz - 2)];
      }
}

/* Pressure-gradient pieces of Projection for one cross direction: returns the
 * cross difference (poisson.c:2370-2411 and the five analogues). */
static inline double cross_diff(int br, double pu0, double pu1, double p0, double p1, double pd0,
                                double pd1) {
  if (br == 2) return (p0 + p1 - pd0 - pd1) * 0.5;
  if (br == 3) return (pu0 + pu1 - p0 - p1) * 0.5;
  if (br == 1) return (pu0 + pu1 - pd0 - pd1) * 0.25;
  return 0.;
}

static void proj_x(const orc_level *L, const double *ph, double dt, double st, double *uc, int i, int j, int k) {
  const int my = L->my, mz = L->mz;
  const int py = L->bctype[2] == 7, pz = L->bctype[4] == 7;
  double dpdc = ph[ID(L, i + 1, j, k)] - ph[ID(L, i, j, k)];
  int bj = cross_branch(NV(L, i, j + 1, k) + NV(L, i + 1, j + 1, k), NV(L, i, j - 1, k) + NV(L, i + 1, j - 1, k), j, my, py);
  double dpde = cross_diff(bj, ph[ID(L, i, j + 1, k)], ph[ID(L, i + 1, j + 1, k)], ph[ID(L, i, j, k)],
                           ph[ID(L, i + 1, j, k)], ph[ID(L, i, j - 1, k)], ph[ID(L, i + 1, j - 1, k)]);
  int bk = cross_branch(NV(L, i, j, k + 1) + NV(L, i + 1, j, k + 1), NV(L, i, j, k - 1) + NV(L, i + 1, j, k - 1), k, mz, pz);
  double dpdz = cross_diff(bk, ph[ID(L, i, j, k + 1)], ph[ID(L, i + 1, j, k + 1)], ph[ID(L, i, j, k)],
                           ph[ID(L, i + 1, j, k)], ph[ID(L, i, j, k - 1)], ph[ID(L, i + 1, j, k - 1)]);
  if (!(NV(L, i, j, k) + NV(L, i + 1, j, k))) {
    size_t p = ID(L, i, j, k);
    const double *ic = L->icsi + 3 * p, *ie = L->ieta + 3 * p, *iz = L->izet + 3 * p;
    double ia = L->iaj[p];
    uc[3 * p] -= (dpdc * dot3(ic, ic) * ia + dpde * dot3(ie, ic) * ia + dpdz * dot3(iz, ic) * ia) * dt * st / COEF;
  }
}

static void proj_y(const orc_level *L, const double *ph, double dt, double st, double *uc, int i, int j, int k) {
  const int mx = L->mx, mz = L->mz;
  const int px = L->bctype[0] == 7, pz = L->bctype[4] == 7;
  int bi = cross_branch(NV(L, i + 1, j, k) + NV(L, i + 1, j + 1, k), NV(L, i - 1, j, k) + NV(L, i - 1, j + 1, k), i, mx, px);
  double dpdc = cross_diff(bi, ph[ID(L, i + 1, j, k)], ph[ID(L, i + 1, j + 1, k)], ph[ID(L, i, j, k)],
                           ph[ID(L, i, j + 1, k)], ph[ID(L, i - 1, j, k)], ph[ID(L, i - 1, j + 1, k)]);
  double dpde = ph[ID(L, i, j + 1, k)] - ph[ID(L, i, j, k)];
  int bk = cross_branch(NV(L, i, j, k + 1) + NV(L, i, j + 1, k + 1), NV(L, i, j, k - 1) + NV(L, i, j + 1, k - 1), k, mz, pz);
  double dpdz = cross_diff(bk, ph[ID(L, i, j, k + 1)], ph[ID(L, i, j + 1, k + 1)], ph[ID(L, i, j, k)],
                           ph[ID(L, i, j + 1, k)], ph[ID(L, i, j, k - 1)], ph[ID(L, i, j + 1, k - 1)]);
  if (!(NV(L, i, j, k) + NV(L, i, j + 1, k))) {
    size_t p = ID(L, i, j, k);
    const double *jc = L->jcsi + 3 * p, *je = L->jeta + 3 * p, *jz = L->jzet + 3 * p;
    double ja = L->jaj[p];
    uc[3 * p + 1] -= (dpdc * dot3(jc, je) * ja + dpde * dot3(je, je) * ja + dpdz * dot3(jz, je) * ja) * dt * st / COEF;
  }
}

static void proj_z(const orc_level *L, const double *ph, double dt, double st, double *uc, int i, int j, int k) {
  const int mx = L->mx, my = L->my;
  const int px = L->bctype[0] == 7, py = L->bctype[2] == 7;
  int bi = cross_branch(NV(L, i + 1, j, k) + NV(L, i + 1, j, k + 1), NV(L, i - 1, j, k) + NV(L, i - 1, j, k + 1), i, mx, px);
  double dpdc = cross_diff(bi, ph[ID(L, i + 1, j, k)], ph[ID(L, i + 1, j, k + 1)], ph[ID(L, i, j, k)],
                           ph[ID(L, i, j, k + 1)], ph[ID(L, i - 1, j, k)], ph[ID(L, i - 1, j, k + 1)]);
  int bj = cross_branch(NV(L, i, j + 1, k) + NV(L, i, j + 1, k + 1), NV(L, i, j - 1, k) + NV(L, i, j - 1, k + 1), j, my, py);
  double dpde = cross_diff(bj, ph[ID(L, i, j + 1, k)], ph[ID(L, i, j + 1, k + 1)], ph[ID(L, i, j, k)],
                           ph[ID(L, i, j, k + 1)], ph[ID(L, i, j - 1, k)], ph[ID(L, i, j - 1, k + 1)]);
  double dpdz = ph[ID(L, i, j, k + 1)] - ph[ID(L, i, j, k)];
  if (!(NV(L, i, j, k) + NV(L, i, j, k + 1))) {
    size_t p = ID(L, i, j, k);
    const double *kc = L->kcsi + 3 * p, *ke = L->keta + 3 * p, *kz = L->kzet + 3 * p;
    double ka = L->kaj[p];
    uc[3 * p + 2] -= (dpdc * dot3(kc, kz) * ka + dpde * dot3(ke, kz) * ka + dpdz * dot3(kz, kz) * ka) * dt * st / COEF;
  }
}

void orc_projection(const orc_level *L, const double *phi, double dt, double st, double *uc) {
  const int mx = L->mx, my = L->my, mz = L->mz;
  const int px = L->bctype[0] == 7, py = L->bctype[2] == 7, pz = L->bctype[4] == 7;
  const int i_end = px ? mx - 1 : mx - 2, j_end = py ? my - 1 : my - 2, k_end = pz ? mz - 1 : mz - 2;
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        if (i < i_end) proj_x(L, phi, dt, st, uc, i, j, k);
        if (j < j_end) proj_y(L, phi, dt, st, uc, i, j, k);
        if (k < k_end) proj_z(L, phi, dt, st, uc, i, j, k);
      }
  if (px)
    for (int k = 1; k < mz - 1; k++)
      for (int j = 1; j < my - 1; j++) proj_x(L, phi, dt, st, uc, 0, j, k);
  if (py)
    for (int k = 1; k < mz - 1; k++)
      for (int i = 1; i < mx - 1; i++) proj_y(L, phi, dt, st, uc, i, 0, k);
  if (pz)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) proj_z(L, phi, dt, st, uc, i, j, 0);
}

/* Contra2Cart (rhs.c:25-143).  Each metric row and flux is the mean of the two
 * faces of the cell; the 3x3 system is solved by Cramer's rule, terms in the
 * reference's order. */
void orc_contra2cart(const orc_level *L, const double *uc, double *ucat) {
  const int mx = L->mx, my = L->my, mz = L->mz;
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        const size_t p = ID(L, i, j, k);
        const double nv = L->nvert[p];
        if (!(nv < 0.1 || nv > 7.0)) continue;
        const size_t pw = ID(L, i - 1, j, k), ps = ID(L, i, j - 1, k), pb = ID(L, i, j, k - 1);
        double m[3][3], q[3];
        for (int c = 0; c < 3; c++) {
          m[0][c] = 0.5 * (L->csi[3 * pw + c] + L->csi[3 * p + c]);
          m[1][c] = 0.5 * (L->eta[3 * ps + c] + L->eta[3 * p + c]);
          m[2][c] = 0.5 * (L->zet[3 * pb + c] + L->zet[3 * p + c]);
        }
        q[0] = 0.5 * (uc[3 * pw + 0] + uc[3 * p + 0]);
        q[1] = 0.5 * (uc[3 * ps + 1] + uc[3 * p + 1]);
        q[2] = 0.5 * (uc[3 * pb + 2] + uc[3 * p + 2]);
        const double det = m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) -
                           m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
                           m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
        const double d0 = q[0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) -
                          q[1] * (m[0][1] * m[2][2] - m[0][2] * m[2][1]) +
                          q[2] * (m[0][1] * m[1][2] - m[0][2] * m[1][1]);
        const double d1 = -q[0] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
                          q[1] * (m[0][0] * m[2][2] - m[0][2] * m[2][0]) -
                          q[2] * (m[0][0] * m[1][2] - m[0][2] * m[1][0]);
        const double d2 = q[0] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]) -
                          q[1] * (m[0][0] * m[2][1] - m[0][1] * m[2][0]) +
                          q[2] * (m[0][0] * m[1][1] - m[0][1] * m[1][0]);
        ucat[3 * p + 0] = d0 / det;
        ucat[3 * p + 1] = d1 / det;
        ucat[3 * p + 2] = d2 / det;
      }
}

/* Slip face (bcs.c:3827-3944): the tangential part of the velocity u next to
 * the face, with n the unit vector of metric m. */
static void slip(const double *m, const double *u, double *ub) {
  const double A = sqrt(m[2] * m[2] + m[1] * m[1] + m[0] * m[0]);
  const double nx = m[0] / A, ny = m[1] / A, nz = m[2] / A;
  const double Un = u[0] * nx + u[1] * ny + u[2] * nz;
  ub[0] = u[0] - Un * nx;
  ub[1] = u[1] - Un * ny;
  ub[2] = u[2] - Un * nz;
}

static inline void copy3(double *d, const double *s) { d[0] = s[0]; d[1] = s[1]; d[2] = s[2]; }
static inline void ghost3(double *g, const double *ub, const double *in) {
  for (int c = 0; c < 3; c++) g[c] = 2 * ub[c] - in[c];
}
static inline void avg3(double *d, const double *a, const double *b) {
  for (int c = 0; c < 3; c++) d[c] = 0.5 * (a[c] + b[c]);
}

int orc_ghost_node_velocity(const orc_level *L, double *ub, double *u) {
  return orc_ghost_node_velocity_ext(L, ub, u, NULL, 0.0);
}

int orc_ghost_node_velocity_ext(const orc_level *L, double *ub, double *u, const double *cent, double u_bc) {
  const int mx = L->mx, my = L->my, mz = L->mz;
  const int *bc = L->bctype;
  const int IM = mx - 1, JM = my - 1, KM = mz - 1;
  if (bc[2] == 11 && !cent) return -1;
  for (int d = 0; d < 3; d++)
    if ((bc[2 * d] == 7) != (bc[2 * d + 1] == 7)) return -1;
#define U3(i, j, k) (u + 3 * ID(L, (i), (j), (k)))
#define B3(i, j, k) (ub + 3 * ID(L, (i), (j), (k)))
  /* boundary velocity of the special wall types (bcs.c:3776-3975); the loops
   * skip the ring of the face */
  if (bc[5] == 2)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        double *b = B3(i, j, mz - 1);
        b[0] = 0.; b[1] = 1.; b[2] = 0.;
      }
  if (bc[3] == 12)
    for (int k = 1; k < mz - 1; k++)
      for (int i = 1; i < mx - 1; i++) {
        double *b = B3(i, my - 1, k);
        b[0] = 0.; b[1] = 0.; b[2] = 1.;
      }
  /* annulus (bctype[2] 11, bcs.c:3811-3825): the tangential unit vector of the
   * cell centre above the face, (y, -x, 0) / |(x, y)| */
  if (bc[2] == 11)
    for (int k = 1; k < mz - 1; k++)
      for (int i = 1; i < mx - 1; i++) {
        const double *c = cent + 3 * ID(L, i, 1, k);
        double *b = B3(i, 0, k);
        b[0] = c[1] / sqrt(c[0] * c[0] + c[1] * c[1]);
        b[1] = -c[0] / sqrt(c[0] * c[0] + c[1] * c[1]);
        b[2] = 0.0;
      }
  if (bc[0] == 3)
    for (int k = 1; k < mz - 1; k++)
      for (int j = 1; j < my - 1; j++) slip(L->csi + 3 * ID(L, 0, j, k), U3(1, j, k), B3(0, j, k));
  if (bc[1] == 3)
    for (int k = 1; k < mz - 1; k++)
      for (int j = 1; j < my - 1; j++)
        slip(L->csi + 3 * ID(L, mx - 2, j, k), U3(mx - 2, j, k), B3(mx - 1, j, k));
  if (bc[2] == 3)
    for (int k = 1; k < mz - 1; k++)
      for (int i = 1; i < mx - 1; i++) slip(L->eta + 3 * ID(L, i, 0, k), U3(i, 1, k), B3(i, 0, k));
  if (bc[3] == 3)
    for (int k = 1; k < mz - 1; k++)
      for (int i = 1; i < mx - 1; i++)
        slip(L->eta + 3 * ID(L, i, my - 2, k), U3(i, my - 2, k), B3(i, my - 1, k));
  /* the k = 0 face takes the velocity of its own (ghost) cell (bcs.c:3918-3926) */
  if (bc[4] == 3)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) slip(L->zet + 3 * ID(L, i, j, 0), U3(i, j, 0), B3(i, j, 0));
  if (bc[5] == 3)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++)
        slip(L->zet + 3 * ID(L, i, j, mz - 2), U3(i, j, mz - 2), B3(i, j, mz - 1));
  /* rheology plates (bctype 13, bcs.c:3963-4010): the plate velocity U_bc */
  if (bc[2] == 13)
    for (int k = 1; k < mz - 1; k++)
      for (int i = 1; i < mx - 1; i++) {
        double *b = B3(i, 0, k);
        b[0] = 0.; b[1] = 0.; b[2] = -u_bc;
      }
  if (bc[3] == 13)
    for (int k = 1; k < mz - 1; k++)
      for (int i = 1; i < mx - 1; i++) {
        double *b = B3(i, my - 1, k);
        b[0] = 0.; b[1] = 0.; b[2] = u_bc;
      }
  if (bc[4] == 13)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        double *b = B3(i, j, 0);
        b[0] = -u_bc; b[1] = 0.; b[2] = 0.;
      }
  if (bc[5] == 13)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        double *b = B3(i, j, mz - 1);
        b[0] = u_bc; b[1] = 0.; b[2] = 0.;
      }
  /* non-periodic ghost faces, whole faces, x then y then z (bcs.c:4015-4076) */
  if (bc[0] != 7)
    for (int k = 0; k < mz; k++)
      for (int j = 0; j < my; j++) {
        ghost3(U3(0, j, k), B3(0, j, k), U3(1, j, k));
        ghost3(U3(mx - 1, j, k), B3(mx - 1, j, k), U3(mx - 2, j, k));
      }
  if (bc[2] != 7)
    for (int k = 0; k < mz; k++)
      for (int i = 0; i < mx; i++) {
        ghost3(U3(i, 0, k), B3(i, 0, k), U3(i, 1, k));
        ghost3(U3(i, my - 1, k), B3(i, my - 1, k), U3(i, my - 2, k));
      }
  if (bc[4] != 7)
    for (int j = 0; j < my; j++)
      for (int i = 0; i < mx; i++) {
        ghost3(U3(i, j, 0), B3(i, j, 0), U3(i, j, 1));
        ghost3(U3(i, j, mz - 1), B3(i, j, mz - 1), U3(i, j, mz - 2));
      }
  /* periodic ring copies, first round: off the box's edges; the upper z face
   * takes only the x component (bcs.c:4083-4170) */
  if (bc[0] == 7)
    for (int k = 1; k < KM; k++)
      for (int j = 1; j < JM; j++) {
        copy3(U3(0, j, k), U3(mx - 2, j, k));
        copy3(U3(mx - 1, j, k), U3(1, j, k));
      }
  if (bc[2] == 7)
    for (int k = 1; k < KM; k++)
      for (int i = 1; i < IM; i++) {
        copy3(U3(i, 0, k), U3(i, my - 2, k));
        copy3(U3(i, my - 1, k), U3(i, 1, k));
      }
  if (bc[4] == 7)
    for (int j = 1; j < JM; j++)
      for (int i = 1; i < IM; i++) {
        copy3(U3(i, j, 0), U3(i, j, mz - 2));
        U3(i, j, mz - 1)[0] = U3(i, j, 1)[0];
      }
  /* the 12 edges, in the reference's order (bcs.c:4176-4283) */
  for (int j = 0; j < my; j++) avg3(U3(0, j, 0), U3(0, j, 1), U3(1, j, 0));
  for (int j = 0; j < my; j++) avg3(U3(mx - 1, j, 0), U3(mx - 1, j, 1), U3(mx - 2, j, 0));
  for (int i = 0; i < mx; i++) avg3(U3(i, 0, 0), U3(i, 0, 1), U3(i, 1, 0));
  for (int i = 0; i < mx; i++) avg3(U3(i, my - 1, 0), U3(i, my - 1, 1), U3(i, my - 2, 0));
  for (int j = 0; j < my; j++) avg3(U3(0, j, mz - 1), U3(0, j, mz - 2), U3(1, j, mz - 1));
  for (int j = 0; j < my; j++) avg3(U3(mx - 1, j, mz - 1), U3(mx - 1, j, mz - 2), U3(mx - 2, j, mz - 1));
  for (int i = 0; i < mx; i++) avg3(U3(i, 0, mz - 1), U3(i, 0, mz - 2), U3(i, 1, mz - 1));
  for (int i = 0; i < mx; i++) avg3(U3(i, my - 1, mz - 1), U3(i, my - 1, mz - 2), U3(i, my - 2, mz - 1));
  for (int k = 0; k < mz; k++) avg3(U3(0, 0, k), U3(0, 1, k), U3(1, 0, k));
  for (int k = 0; k < mz; k++) avg3(U3(mx - 1, 0, k), U3(mx - 1, 1, k), U3(mx - 2, 0, k));
  for (int k = 0; k < mz; k++) avg3(U3(0, my - 1, k), U3(0, my - 2, k), U3(1, my - 1, k));
  for (int k = 0; k < mz; k++) avg3(U3(mx - 1, my - 1, k), U3(mx - 1, my - 2, k), U3(mx - 2, my - 1, k));
  /* second round over whole faces, x, then y, then z; the upper z face again
   * only the x component (bcs.c:4287-4405) */
  if (bc[0] == 7)
    for (int k = 0; k < mz; k++)
      for (int j = 0; j < my; j++) {
        copy3(U3(0, j, k), U3(mx - 2, j, k));
        copy3(U3(mx - 1, j, k), U3(1, j, k));
      }
  if (bc[2] == 7)
    for (int k = 0; k < mz; k++)
      for (int i = 0; i < mx; i++) {
        copy3(U3(i, 0, k), U3(i, my - 2, k));
        copy3(U3(i, my - 1, k), U3(i, 1, k));
      }
  if (bc[4] == 7)
    for (int j = 0; j < my; j++)
      for (int i = 0; i < mx; i++) {
        copy3(U3(i, j, 0), U3(i, j, mz - 2));
        U3(i, j, mz - 1)[0] = U3(i, j, 1)[0];
      }
#undef U3
#undef B3
  return 0;
}

/* ------------------------------------------------------------------ IB search */
/* intsect_triangle (compgeom.c:17-50): the ray orig + t dir against one
 * triangle; 1 with (t, u, v) on a hit. */
static int ray_triangle(const double *o, const double *d, const double *v0, const double *v1, const double *v2,
                        double *t) {
  double e1[3], e2[3], pv[3], tv[3], qv[3];
  for (int c = 0; c < 3; c++) { e1[c] = v1[c] - v0[c]; e2[c] = v2[c] - v0[c]; }
  pv[0] = d[1] * e2[2] - d[2] * e2[1];
  pv[1] = d[2] * e2[0] - d[0] * e2[2];
  pv[2] = d[0] * e2[1] - d[1] * e2[0];
  const double det = e1[0] * pv[0] + e1[1] * pv[1] + e1[2] * pv[2];
  if (det > -0.00000001 && det < 0.00000001) return 0;
  const double inv = 1.0 / det;
  for (int c = 0; c < 3; c++) tv[c] = o[c] - v0[c];
  const double u = (tv[0] * pv[0] + tv[1] * pv[1] + tv[2] * pv[2]) * inv;
  if (u < 0.0 || u > 1.0) return 0;
  qv[0] = tv[1] * e1[2] - tv[2] * e1[1];
  qv[1] = tv[2] * e1[0] - tv[0] * e1[2];
  qv[2] = tv[0] * e1[1] - tv[1] * e1[0];
  const double v = (d[0] * qv[0] + d[1] * qv[1] + d[2] * qv[2]) * inv;
  if (v < 0.0 || u + v > 1.0) return 0;
  *t = (e2[0] * qv[0] + e2[1] * qv[1] + e2[2] * qv[2]) * inv;
  return 1;
}

enum { IBM_NC = 40, IBM_MAX_HITS = 1000 };

typedef struct {
  double min[3], max[3], dc[3];
  int *col_start, *col_tri, *col_jmax;  /* bucket column (i, k) -> triangles and their j range end */
} ibm_grid;

static void ibm_grid_build(ibm_grid *G, int n_v, const double *xyz, int n_elmt, const int *tri) {
  for (int c = 0; c < 3; c++) { G->min[c] = 1.e23; G->max[c] = -1.e23; }
  for (int q = 0; q < n_v; q++)
    for (int c = 0; c < 3; c++) {
      const double x = xyz[3 * q + c];
      G->min[c] = G->min[c] < x ? G->min[c] : x;
      G->max[c] = G->max[c] < x ? x : G->max[c];
    }
  for (int c = 0; c < 3; c++) G->dc[c] = (G->max[c] - G->min[c]) / (IBM_NC - 1.);
  /* bucket ranges of every triangle (ibm.c:4279-4318), then the lists of the
   * (i, k) columns: a ray from bucket j walks the column's buckets j .. NC-1,
   * so it meets the triangles whose j range ends above j */
  int (*rng)[6] = malloc(sizeof(int[6]) * (size_t)(n_elmt > 0 ? n_elmt : 1));
  G->col_start = calloc(IBM_NC * IBM_NC + 1, sizeof(int));
  for (int e = 0; e < n_elmt; e++) {
    for (int c = 0; c < 3; c++) {
      const double a = xyz[3 * tri[3 * e] + c], b = xyz[3 * tri[3 * e + 1] + c], d = xyz[3 * tri[3 * e + 2] + c];
      double lo = a < b ? a : b, hi = a < b ? b : a;
      lo = lo < d ? lo : d;
      hi = hi < d ? d : hi;
      int imin = (int)floor((lo - G->min[c]) / G->dc[c]);
      int imax = (int)floor((hi - G->min[c]) / G->dc[c]) + 1;
      rng[e][2 * c] = imin < 0 ? 0 : imin;
      rng[e][2 * c + 1] = imax > IBM_NC ? IBM_NC : imax;
    }
    for (int k = rng[e][4]; k < rng[e][5]; k++)
      for (int i = rng[e][0]; i < rng[e][1]; i++)
        if (rng[e][2] < rng[e][3]) G->col_start[k * IBM_NC + i + 1]++;
  }
  for (int q = 0; q < IBM_NC * IBM_NC; q++) G->col_start[q + 1] += G->col_start[q];
  const int total = G->col_start[IBM_NC * IBM_NC];
  G->col_tri = malloc(sizeof(int) * (size_t)(total > 0 ? total : 1));
  G->col_jmax = malloc(sizeof(int) * (size_t)(total > 0 ? total : 1));
  int *fill = calloc(IBM_NC * IBM_NC, sizeof(int));
  for (int e = 0; e < n_elmt; e++) {
    if (rng[e][2] >= rng[e][3]) continue;
    for (int k = rng[e][4]; k < rng[e][5]; k++)
      for (int i = rng[e][0]; i < rng[e][1]; i++) {
        const int col = k * IBM_NC + i, at = G->col_start[col] + fill[col]++;
        G->col_tri[at] = e;
        G->col_jmax[at] = rng[e][3];
      }
  }
  free(fill);
  free(rng);
}

/* point_cell_advanced (ibm.c:1285-1400) with randomdirection (ibm.c:87-118):
 * 4 when p is inside the body, else 0; -1 when max_tries rays all met a
 * singular pair (two hits at the same distance on faces not facing apart). */
static int point_inside(const ibm_grid *G, const double *p, int ic, int jc, int kc, const double *xyz, const int *tri,
                        const double *nf, int max_tries) {
  static double dt[IBM_MAX_HITS], dn[IBM_MAX_HITS][3];
  const int col = kc * IBM_NC + ic;
  for (int seed = 1; seed <= max_tries; seed++) {
    const double xpc = G->dc[0] * (ic + 0.5) + G->min[0];
    const double zpc = G->dc[2] * (kc + 0.5) + G->min[2];
    srand(seed);
    double s = rand() / ((double)RAND_MAX + 1) - 0.5;
    double d[3];
    d[0] = (xpc + s * G->dc[0]) - p[0];
    d[1] = (G->max[1] + 0.2) - p[1];
    d[2] = (zpc + s * G->dc[2]) - p[2];
    s = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    d[0] /= s; d[1] /= s; d[2] /= s;
    int hits = 0, singular = 0;
    for (int q = G->col_start[col]; q < G->col_start[col + 1] && !singular; q++) {
      if (G->col_jmax[q] <= jc) continue;
      const int e = G->col_tri[q];
      double t;
      if (!ray_triangle(p, d, xyz + 3 * tri[3 * e], xyz + 3 * tri[3 * e + 1], xyz + 3 * tri[3 * e + 2], &t)) continue;
      if (!(t > 0)) continue;
      const double *n = nf + 3 * e;
      if (hits == IBM_MAX_HITS) return -1;
      for (int h = 0; h < hits; h++) {
        const double ndotn = dn[h][0] * n[0] + dn[h][1] * n[1] + dn[h][2] * n[2];
        if (fabs(t - dt[h]) < 1.e-8 && ndotn > -0.97) singular = 1;
      }
      dt[hits] = t;
      dn[hits][0] = n[0]; dn[hits][1] = n[1]; dn[hits][2] = n[2];
      hits++;
    }
    if (!singular) return (hits % 2) ? 4 : 0;
  }
  return -1;
}

int orc_ibm_search(int mx, int my, int mz, const double *cent, int n_v, const double *xyz, int n_elmt,
                   const int *tri, const double *nf, int ibi, int nbodies, const double *nvert_o, double *nvert,
                   int max_tries) {
  ibm_grid G;
  ibm_grid_build(&G, n_v, xyz, n_elmt, tri);
  const size_t n = (size_t)mx * my * mz;
  double *nv = malloc(sizeof(double) * n);
  memcpy(nv, nvert, sizeof(double) * n);
  int rc = 0;
#define P(i, j, k) (((size_t)(k) * my + (j)) * mx + (i))
  /* the inside test on interior cells (ibm.c:4337-4357) */
  for (int k = 1; k < mz - 1 && !rc; k++)
    for (int j = 1; j < my - 1 && !rc; j++)
      for (int i = 1; i < mx - 1 && !rc; i++) {
        const size_t q = P(i, j, k);
        if (ibi == 0 && nv[q] < 5.) nv[q] = 0;
        const double *c = cent + 3 * q;
        if (c[0] > G.min[0] && c[0] < G.max[0] && c[1] > G.min[1] && c[1] < G.max[1] && c[2] > G.min[2] &&
            c[2] < G.max[2]) {
          const int ic = (int)floor((c[0] - G.min[0]) / G.dc[0]);
          const int jc = (int)floor((c[1] - G.min[1]) / G.dc[1]);
          const int kc = (int)floor((c[2] - G.min[2]) / G.dc[2]);
          const int r = point_inside(&G, c, ic, jc, kc, xyz, tri, nf, max_tries);
          if (r < 0) { rc = -1; break; }
          if (nv[q] < r) nv[q] = r;
          if (nv[q] < 0) nv[q] = 0;
        }
      }
  if (!rc) {
    /* the layer: every cell next to an inside cell (ibm.c:4415-4437); no cell
     * becomes inside here, so reading the updated array changes nothing */
    for (int k = 0; k < mz; k++)
      for (int j = 0; j < my; j++)
        for (int i = 0; i < mx; i++) {
          const size_t q = P(i, j, k);
          if (nv[q] < 0) nv[q] = 0;
          if ((int)(nv[q] + 0.5) == 4) continue;
          const int ip = i < mx - 1 ? i + 1 : i, im = i > 0 ? i - 1 : i;
          const int jp = j < my - 1 ? j + 1 : j, jm = j > 0 ? j - 1 : j;
          const int kp = k < mz - 1 ? k + 1 : k, km = k > 0 ? k - 1 : k;
          for (int kk = km; kk <= kp; kk++)
            for (int jj = jm; jj <= jp; jj++)
              for (int ii = im; ii <= ip; ii++)
                if ((int)(nv[P(ii, jj, kk)] + 0.5) == 4) nv[q] = 2 < nv[q] ? nv[q] : 2;
        }
    /* a solid cell of the previous step that the search left fluid (ibm.c:4499-4509) */
    if (ibi == nbodies - 1)
      for (size_t q = 0; q < n; q++)
        if (nvert_o[q] > 2.5 && nv[q] < 0.5) nv[q] = 2;
    /* this body's codes (ibm.c:4651-4659) */
    for (size_t q = 0; q < n; q++) {
      if ((int)(nv[q] + 0.5) == 2) nv[q] = 1 + (ibi) / 1000.0;
      if ((int)(nv[q] + 0.5) == 4) nv[q] = 3 + (ibi) / 1000.0;
    }
    /* an IB cell between two fluid cells in k becomes fluid, twice
     * (ibm.c:4662-4690), in the reference's order */
    for (int pass = 0; pass < 2; pass++)
      for (int k = 1; k < mz - 1; k++)
        for (int j = 1; j < my - 1; j++)
          for (int i = 1; i < mx - 1; i++) {
            const size_t q = P(i, j, k);
            int around = 0;
            if ((int)(nv[q]) == 1) {
              if ((int)(nv[P(i, j, k - 1)]) == 0) around++;
              if ((int)(nv[P(i, j, k + 1)]) == 0) around++;
            }
            if (around > 1) nv[q] = 0 < nv[q] ? 0 : nv[q];
          }
    memcpy(nvert, nv, sizeof(double) * n);
  }
#undef P
  free(nv);
  free(G.col_start); free(G.col_tri); free(G.col_jmax);
  return rc;
}

void orc_ibm_ray_offsets(int n, double *s) {
  for (int q = 0; q < n; q++) {
    srand(q + 1);
    s[q] = rand() / ((double)RAND_MAX + 1) - 0.5;
  }
}

void orc_divergence(const orc_level *L, const double *uc, double *maxdiv, long long *at) {
  const int mx = L->mx, my = L->my, mz = L->mz;
  double m = -HUGE_VAL;
  long long where = -1;
  for (int k = 0; k < mz; k++)
    for (int j = 0; j < my; j++)
      for (int i = 0; i < mx; i++) {
        double d = 0.0;
        if (i > 0 && i < mx - 1 && j > 0 && j < my - 1 && k > 0 && k < mz - 1) {
          const size_t p = ID(L, i, j, k);
          const size_t w = ID(L, i - 1, j, k), s = ID(L, i, j - 1, k), b = ID(L, i, j, k - 1);
          d = fabs((uc[3 * p] - uc[3 * w] + uc[3 * p + 1] - uc[3 * s + 1] + uc[3 * p + 2] - uc[3 * b + 2]) * L->aj[p]);
          if (NV(L, i, j, k) + NV(L, i, j, k + 1) + NV(L, i, j, k - 1) + NV(L, i, j + 1, k) + NV(L, i, j - 1, k) +
                  NV(L, i + 1, j, k) + NV(L, i - 1, j, k) > 0.1)
            d = 0.;
        }
        if (d > m) { m = d; where = (long long)ID(L, i, j, k); }
      }
  *maxdiv = m;
  *at = where;
}

/* One face flux component of Convection (rhs.c:1628-1918): lo is the offset of
 * the upwind cell below (-1 interior, 0 next to the low end), hi the one above
 * (2 interior, 1 next to the high end), st the stride along the direction. */
static double conv_quick(const double *uc, size_t p, long st, int c, int lo, int hi, double um, double up) {
  const double coef = 0.125;
#define UC(o) uc[3 * (size_t)((long)p + (long)(o) * st) + c]
  return um * (coef * (-UC(hi) - 2. * UC(1) + 3. * UC(0)) + UC(1)) +
         up * (coef * (-UC(lo) - 2. * UC(0) + 3. * UC(1)) + UC(0));
#undef UC
}

static int conv_fluid(double n) { return n < 0.1 || n > 7.; }

int orc_convection(const orc_level *L, const double *ucont, const double *ucat, int central, double *conv) {
  const int mx = L->mx, my = L->my, mz = L->mz;
  /* a periodic direction: the reference first sets the ghost cells just
   * outside the box to the images two cells further out (rhs.c:1546-1620):
   * index -1 reads m - 3, index m reads 2 (ucat and nvert alike) */
  const int per[3] = {L->bctype[0] == 7 || L->bctype[1] == 7, L->bctype[2] == 7 || L->bctype[3] == 7,
                      L->bctype[4] == 7 || L->bctype[5] == 7};
  const size_t n = (size_t)mx * my * mz;
  const long st[3] = {1, mx, (long)mx * my};
  const int ext[3] = {mx, my, mz};
  double *fp = (double *)calloc(9 * n, sizeof(double));
  for (int d = 0; d < 3; d++)
    for (int k = d == 2 ? 0 : 1; k < mz - 1; k++)
      for (int j = d == 1 ? 0 : 1; j < my - 1; j++)
        for (int i = d == 0 ? 0 : 1; i < mx - 1; i++) {
          const size_t p = ID(L, i, j, k);
          const int q = d == 0 ? i : d == 1 ? j : k, m = ext[d];
          const double *nv = L->nvert;
          const double ucon = ucont[3 * p + d] * 0.5;
          const double up = ucon + fabs(ucon), um = ucon - fabs(ucon);
          double *o = fp + 9 * p + 3 * d;
#define NV(off) nv[(size_t)((long)p + (long)(off) * st[d])]
#define UC(off, c) ucat[3 * (size_t)((long)p + (long)(off) * st[d]) + c]
          int lo = 0, hi = 0, cen = 0;
          /* the j sweep tests i (not j) against my-2 for its central end faces */
          const int end2 = d == 1 ? (j == 0 || i == my - 2) : (q == 0 || q == m - 2);
          if (q > 0 && q < m - 2 && conv_fluid(NV(1)) && conv_fluid(NV(-1))) {
            if (central) cen = 1; else { lo = -1; hi = 2; }
          } else if (central && end2 && conv_fluid(NV(1)) && conv_fluid(NV(0))) {
            cen = 1;
          } else if ((d < 2 || q < m - 2) && (q == 0 || NV(-1) > 0.1)) {
            /* periodic low end with fluid on both sides: the full QUICK form
             * across the seam (rhs.c:1675-1685 and its j, k siblings) */
            if (per[d] && q == 0 && NV(m - 3) < 0.1 && NV(1) < 0.1) { lo = m - 3; hi = 2; }
            else { lo = 0; hi = 2; }
          } else if ((d < 2 || q > 0) && (q == m - 2 || NV(1) > 0.1)) {
            if (per[d] && q == m - 2 && NV(-1) < 0.1 && NV(1) < 0.1) { lo = -1; hi = 4 - m; }
            else { lo = -1; hi = 1; }
          } else {
            continue;
          }
          for (int c = 0; c < 3; c++)
            o[c] = cen ? ucon * (UC(0, c) + UC(1, c)) : conv_quick(ucat, p, st[d], c, lo, hi, um, up);
#undef NV
#undef UC
        }
  memset(conv, 0, sizeof(double) * 3 * n);
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        const size_t p = ID(L, i, j, k), w = p - 1, s = p - mx, b = p - (size_t)mx * my;
        for (int c = 0; c < 3; c++)
          conv[3 * p + c] = fp[9 * p + c] - fp[9 * w + c] + fp[9 * p + 3 + c] - fp[9 * s + 3 + c] +
                            fp[9 * p + 6 + c] - fp[9 * b + 6 + c];
      }
  free(fp);
  return 0;
}

void orc_metrics_divergence(const orc_level *L, double *maxdiv, long long *at) {
  const int mx = L->mx, my = L->my, mz = L->mz;
  const double *cs = L->csi, *et = L->eta, *ze = L->zet;
  double m = -HUGE_VAL;
  long long where = -1;
  for (int k = 0; k < mz; k++)
    for (int j = 0; j < my; j++)
      for (int i = 0; i < mx; i++) {
        double d = 0.0;
        if (i > 0 && i < mx - 1 && j > 0 && j < my - 1 && k > 0 && k < mz - 1) {
          const size_t p = ID(L, i, j, k);
          const size_t w = ID(L, i - 1, j, k), s = ID(L, i, j - 1, k), b = ID(L, i, j, k - 1);
          double sum = 0.0;
          for (int c = 0; c < 3; c++) {
            const double t = c == 0 ? cs[3 * p] - cs[3 * w] : sum + cs[3 * p + c] - cs[3 * w + c];
            sum = t + et[3 * p + c] - et[3 * s + c] + ze[3 * p + c] - ze[3 * b + c];
          }
          d = fabs(sum * L->aj[p]);
        }
        if (d > m) { m = d; where = (long long)ID(L, i, j, k); }
      }
  *maxdiv = m;
  *at = where;
}

/* ------------------------------------------------------------------ momentum
 * Viscous (rhs.c:1947-2566), laminar (no LES/RANS model, no Clark term): the
 * viscous flux nu (G grad u) on every cell face, then its differences over
 * each interior cell; the ring of visc is 0 (VecSet).  Face d of cell P lies
 * between P and P + e_d; its tangential derivatives are one-sided next to cells
 * with nvert in (0.5, 7) (rhs.c:2056-2110).  Operation order as the reference's. */
static int visc_blocked(double n) { return n > 0.5 && n < 7.; }

void orc_viscous(const orc_level *L, const double *ucat, double ren, double *visc) {
  const int mx = L->mx, my = L->my, mz = L->mz;
  const size_t n = (size_t)mx * my * mz;
  const long st[3] = {1, mx, (long)mx * my};
  const double *mi[3][3] = {{L->icsi, L->ieta, L->izet}, {L->jcsi, L->jeta, L->jzet}, {L->kcsi, L->keta, L->kzet}};
  const double *fa[3] = {L->iaj, L->jaj, L->kaj};
  const double nu = 1. / ren;
  double *fp = (double *)calloc(9 * n, sizeof(double));
  for (int d = 0; d < 3; d++)
    for (int k = d == 2 ? 0 : 1; k < mz - 1; k++)
      for (int j = d == 1 ? 0 : 1; j < my - 1; j++)
        for (int i = d == 0 ? 0 : 1; i < mx - 1; i++) {
          const long p = (long)ID(L, i, j, k), sd = st[d];
          double D[3][3]; /* D[a][c]: derivative of component c along direction a */
          for (int c = 0; c < 3; c++) D[d][c] = ucat[3 * (p + sd) + c] - ucat[3 * p + c];
          for (int t = 0; t < 3; t++) {
            if (t == d) continue;
            const long s = st[t];
            const double *nv = L->nvert;
            const int up = visc_blocked(nv[p + s]) || visc_blocked(nv[p + sd + s]);
            const int dn = visc_blocked(nv[p - s]) || visc_blocked(nv[p + sd - s]);
            for (int c = 0; c < 3; c++) {
#define U(off) ucat[3 * (p + (off)) + c]
              if (up) D[t][c] = (U(sd) + U(0) - U(sd - s) - U(-s)) * 0.5;
              else if (dn) D[t][c] = (U(sd + s) + U(s) - U(sd) - U(0)) * 0.5;
              else D[t][c] = (U(sd + s) + U(s) - U(sd - s) - U(-s)) * 0.25;
#undef U
            }
          }
          const double *m[3] = {mi[d][0] + 3 * p, mi[d][1] + 3 * p, mi[d][2] + 3 * p}; /* csi, eta, zet */
          const double *nd = m[d];
          double g[3];
          for (int a = 0; a < 3; a++) g[a] = m[a][0] * nd[0] + m[a][1] * nd[1] + m[a][2] * nd[2];
          double r[3][3]; /* r[q][c]: grad of component q against metric component c */
          for (int q = 0; q < 3; q++)
            for (int c = 0; c < 3; c++) r[q][c] = D[0][q] * m[0][c] + D[1][q] * m[1][c] + D[2][q] * m[2][c];
          const double ajc = fa[d][p];
          for (int c = 0; c < 3; c++) {
            double v = 0;
            v += (g[0] * D[0][c] + g[1] * D[1][c] + g[2] * D[2][c] + r[0][c] * nd[0] + r[1][c] * nd[1] +
                  r[2][c] * nd[2]) * ajc * (nu);
            fp[9 * p + 3 * d + c] = v;
          }
        }
  memset(visc, 0, sizeof(double) * 3 * n);
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        const size_t p = ID(L, i, j, k), w = p - 1, s = p - mx, b = p - (size_t)mx * my;
        for (int c = 0; c < 3; c++)
          visc[3 * p + c] = (fp[9 * p + c] - fp[9 * w + c] + fp[9 * p + 3 + c] - fp[9 * s + 3 + c] +
                             fp[9 * p + 6 + c] - fp[9 * b + 6 + c]);
      }
  free(fp);
}

/* One of FormFunction1's tangential pressure derivatives at face d of cell P
 * (rhs.c:2803-2849 and its five siblings), walled boxes: one-sided next to a
 * wall or a blocked pair of cells, central otherwise.  Returns 0 where the
 * reference assigns nothing (the variable then keeps its previous value). */
static int ff_dp(const orc_level *L, const double *p, long P, long sd, long s, int q, int m, double *val) {
  const double *nv = L->nvert;
  const double up = nv[P + s] + nv[P + sd + s], dn = nv[P - s] + nv[P + sd - s];
  if (q == m - 2 || up > 0.1) {
    if (dn < 0.1 && q != 1) {
      *val = (p[P] + p[P + sd] - p[P - s] - p[P + sd - s]) * 0.5;
      return 1;
    }
    return 0;
  }
  if (q == 1 || dn > 0.1) {
    if (up < 0.1) {
      *val = (p[P + s] + p[P + sd + s] - p[P] - p[P + sd]) * 0.5;
      return 1;
    }
    return 0;
  }
  *val = (p[P + s] + p[P + sd + s] - p[P - s] - p[P + sd - s]) * 0.25;
  return 1;
}

/* FormFunction1 (rhs.c:2567-3351) for a box with no periodic face: Contra2Cart
 * (ucat's interior cells from ucont), Convection, Viscous, rc = visc - conv,
 * its contravariant form rct at the cell centres, then on every face the
 * average of rct minus the pressure gradient (G grad p) and the blocked-face
 * masks.  rhs ([mz][my][mx][3]) is written on the interior cells only.  The
 * pressure derivatives keep the reference's loop order: where a branch assigns
 * nothing, the value of the previous assignment in that order stands (the
 * reference leaves the variables uninitialised before the first cell; they
 * start at 0 here).  Returns -1 for a periodic box. */
int orc_form_function1(const orc_level *L, const double *ucont, double *ucat, const double *p, double ren,
                       int central, double *rhs) {
  const int mx = L->mx, my = L->my, mz = L->mz;
  for (int f = 0; f < 6; f++)
    if (L->bctype[f] == 7) return -1;
  const size_t n = (size_t)mx * my * mz;
  orc_contra2cart(L, ucont, ucat);
  double *conv = (double *)malloc(sizeof(double) * 3 * n), *visc = (double *)malloc(sizeof(double) * 3 * n);
  double *rct = (double *)calloc(3 * n, sizeof(double));
  orc_convection(L, ucont, ucat, central, conv);
  orc_viscous(L, ucat, ren, visc);
  const long sx = 1, sy = mx, sz = (long)mx * my;
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        const long P = (long)ID(L, i, j, k);
        double rc[3];
        for (int c = 0; c < 3; c++) rc[c] = -1.0 * conv[3 * P + c] + visc[3 * P + c];
        const double *cs = L->csi, *et = L->eta, *ze = L->zet;
        const double a = L->aj[P];
        rct[3 * P + 0] = a * (0.5 * (cs[3 * P] + cs[3 * (P - sx)]) * rc[0] +
                              0.5 * (cs[3 * P + 1] + cs[3 * (P - sx) + 1]) * rc[1] +
                              0.5 * (cs[3 * P + 2] + cs[3 * (P - sx) + 2]) * rc[2]);
        rct[3 * P + 1] = a * (0.5 * (et[3 * P] + et[3 * (P - sy)]) * rc[0] +
                              0.5 * (et[3 * P + 1] + et[3 * (P - sy) + 1]) * rc[1] +
                              0.5 * (et[3 * P + 2] + et[3 * (P - sy) + 2]) * rc[2]);
        rct[3 * P + 2] = a * (0.5 * (ze[3 * P] + ze[3 * (P - sz)]) * rc[0] +
                              0.5 * (ze[3 * P + 1] + ze[3 * (P - sz) + 1]) * rc[1] +
                              0.5 * (ze[3 * P + 2] + ze[3 * (P - sz) + 2]) * rc[2]);
      }
  double dpdc = 0.0, dpde = 0.0, dpdz = 0.0;
  const double *fm[3][3] = {{L->icsi, L->ieta, L->izet}, {L->jcsi, L->jeta, L->jzet}, {L->kcsi, L->keta, L->kzet}};
  const double *fa[3] = {L->iaj, L->jaj, L->kaj};
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        const long P = (long)ID(L, i, j, k);
        const long st[3] = {sx, sy, sz};
        for (int d = 0; d < 3; d++) {
          double *dp[3] = {&dpdc, &dpde, &dpdz};
          const int q[3] = {i, j, k}, m[3] = {mx, my, mz};
          for (int t = 0; t < 3; t++) {
            if (t == d) *dp[t] = p[P + st[d]] - p[P];
            else ff_dp(L, p, P, st[d], st[t], q[t], m[t], dp[t]);
          }
          const double *cs = fm[d][0] + 3 * P, *et = fm[d][1] + 3 * P, *zt = fm[d][2] + 3 * P;
          const double *nd = d == 0 ? cs : d == 1 ? et : zt;
          double v = 0.5 * (rct[3 * P + d] + rct[3 * (P + st[d]) + d]);
          v -= (dpdc * (cs[0] * nd[0] + cs[1] * nd[1] + cs[2] * nd[2]) +
                dpde * (et[0] * nd[0] + et[1] * nd[1] + et[2] * nd[2]) +
                dpdz * (zt[0] * nd[0] + zt[1] * nd[1] + zt[2] * nd[2])) * fa[d][P];
          rhs[3 * P + d] = v;
        }
      }
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        const long P = (long)ID(L, i, j, k);
        const double *nv = L->nvert;
        if (nv[P] > 0.1) rhs[3 * P] = rhs[3 * P + 1] = rhs[3 * P + 2] = 0;
        if (nv[P + sx] > 0.1) rhs[3 * P] = 0;
        if (nv[P + sy] > 0.1) rhs[3 * P + 1] = 0;
        if (nv[P + sz] > 0.1) rhs[3 * P + 2] = 0;
      }
  free(conv);
  free(visc);
  free(rct);
  return 0;
}

/* CalcRHS (implicitsolver.c:6449-6713) for a box with no periodic face:
 * FormFunction1, the time derivative subtracted -- second-order backward
 * (1.5 u - 2 u_o + 0.5 u_rm1, COEF_TIME_ACCURACY 1.5, variables.h:421) unless
 * this is the first step (ti == tistart or ti == 1), then u - u_o -- divided
 * by dt over every entry, the faces next to blocked cells and the walls
 * zeroed, the convective-outflow term on the last k face when bctype[5] is 8,
 * and the boundary ring zeroed as the reference's six boundary loops do. */
int orc_calc_rhs(const orc_level *L, const double *ucont, const double *ucont_o, const double *ucont_rm1,
                 double *ucat, const double *p, double ren, double dt, int ti, int tistart, int central,
                 double *rhs) {
  const int mx = L->mx, my = L->my, mz = L->mz;
  if (orc_form_function1(L, ucont, ucat, p, ren, central, rhs)) return -1;
  const size_t n3 = 3 * (size_t)mx * my * mz;
  double *du = (double *)malloc(sizeof(double) * n3);
  if (1.5 > 1.1 && ti != tistart && ti != 1) {
    memcpy(du, ucont, sizeof(double) * n3);
    for (size_t q = 0; q < n3; q++) du[q] *= 1.5;
    for (size_t q = 0; q < n3; q++) du[q] += -2. * ucont_o[q];
    for (size_t q = 0; q < n3; q++) du[q] += 0.5 * ucont_rm1[q];
  } else {
    for (size_t q = 0; q < n3; q++) du[q] = -1. * ucont_o[q] + ucont[q];
  }
  const double a = -1. / dt;
  for (size_t q = 0; q < n3; q++) rhs[q] += a * du[q];
  free(du);
  const double c = 0.8;
  const int mz_end = L->bctype[5] == 8 ? mz - 2 : mz - 3;
  const long sx = 1, sy = mx, sz = (long)mx * my;
  const double *nv = L->nvert;
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        const long P = (long)ID(L, i, j, k);
        if ((nv[P] + nv[P + sx]) > 0.1 || i > mx - 3) rhs[3 * P] = 0.;
        if ((nv[P] + nv[P + sy]) > 0.1 || j > my - 3) rhs[3 * P + 1] = 0.;
        if ((nv[P] + nv[P + sz]) > 0.1 || k > mz_end) rhs[3 * P + 2] = 0.;
        if (mz_end == mz - 2 && k == mz - 2) rhs[3 * P + 2] += c * (ucont[3 * P + 2] - ucont[3 * (P - sz) + 2]);
      }
#define R3(i, j, k) (rhs + 3 * ID(L, i, j, k))
  for (int k = 0; k < mz - 1; k++)
    for (int j = 0; j < my - 1; j++) {
      double *r = R3(0, j, k);
      r[0] = r[1] = r[2] = 0;
      R3(mx - 2, j, k)[0] = 0;
      r = R3(mx - 1, j, k);
      r[0] = r[1] = r[2] = 0;
    }
  for (int k = 0; k < mz - 1; k++)
    for (int i = 0; i < mx - 1; i++) {
      double *r = R3(i, 0, k);
      r[0] = r[1] = r[2] = 0;
      R3(i, my - 2, k)[1] = 0;
      r = R3(i, my - 1, k);
      r[0] = r[1] = r[2] = 0;
    }
  for (int j = 0; j < my - 1; j++)
    for (int i = 0; i < mx - 1; i++) {
      double *r = R3(i, j, 0);
      r[0] = r[1] = r[2] = 0;
      R3(i, j, mz - 2)[2] = 0;
      r = R3(i, j, mz - 1);
      r[0] = r[1] = r[2] = 0;
    }
#undef R3
  return 0;
}

/* ------------------------------------------------------------------------ */
/* The momentum equation's pseudo-time iteration, one block, no immersed-body
 * interpolation (immersed 0), for boxes whose x and y faces are solid walls
 * (bctype 1) and whose k = 0 and k = mz - 1 faces are walls or an inlet
 * (bctype[4] 5) and an outlet (bctype[5] 4). */

/* The inlet speed of InflowFlux's constant profiles (bcs.c:161-200); 0 for
 * the profiles that are not restated. */
/* The reference's Flux_in (main.c:6, its initial value) and ti globals, which
 * profiles 3, 6 and 8 read (bcs.c:67-82). */
static double g_flux_in = 4.104388e-04;
static int g_ti = 0;
void orc_set_inlet_globals(double flux_in, int ti) {
  g_flux_in = flux_in;
  g_ti = ti;
}

int orc_inlet_speed(int inletprofile, double *uin) {
  if (inletprofile == 1) *uin = 2.;
  else if (inletprofile == -1) *uin = -1.;
  else if (inletprofile == 11) *uin = 0.185;
  else if (inletprofile == 3 || inletprofile == 6) *uin = g_flux_in;
  else if (inletprofile == 8) *uin = g_flux_in = sin(2 * 3.14159 * g_ti / 200.); /* and Flux_in keeps it */
  else return 0;
  return 1;
}

int orc_bcs_covered(const int *bc) {
  for (int f = 0; f < 4; f++)
    if (bc[f] != 1) return 0;
  if (bc[4] != 1 && bc[4] != 5) return 0;
  if (bc[5] != 1 && bc[5] != 4) return 0;
  return (bc[5] == 4) == (bc[4] == 5);
}

/* InletInterpolation's table (bcs.c:67-96): uinr [101][1001] of InletRead
 * (bcs.c:40-55; radius r[i] = 0.005 i, one column per time step), at the
 * step tstep = ti / 2 - (ti / 2000) 2000; beyond r = 1 the speed of r[99],
 * between r[100] and 1 zero. */
static const double *g_inlet_table;
void orc_set_inlet_table(const double *uinr) { g_inlet_table = uinr; }
static int table_step_ok(void) {
  const int tstep = g_ti / 2 - ((g_ti / 2000) * 2000);
  return g_inlet_table && tstep >= 0 && tstep < 1001;
}
static double table_speed(double r) {
  const int tstep = g_ti / 2 - ((g_ti / 2000) * 2000);
  const double *U = g_inlet_table + tstep;
  if (r > 1.) return U[99 * 1001];
  for (int i = 0; i < 100; i++) {
    const double ri = i * 0.005, ri1 = (i + 1) * 0.005;
    if (r >= ri && r < ri1) return U[i * 1001] + (U[(i + 1) * 1001] - U[i * 1001]) * (r - ri) / (ri1 - ri);
  }
  return 0;
}

/* Profile 10 (bcs.c:180-195): fully developed laminar flow in a square duct
 * (y across [1, 2], x across [0, 1] about the centre), 1 - y'^2 less the
 * first 20 terms of its Fourier series in y' = 2 (y - 1.5), x' = x - 0.5;
 * each term's factors multiplied and divided left to right, through libm's
 * pow, cosh and cos. */
double orc_duct_speed(double xc, double yc) {
  const double pi = 3.14159265358979323846264338327950288;
  const double y = (yc - 1.5) * 2., x = xc - 0.5, A = 1.;
  double u = 1 - y * y;
  for (int n = 0; n < 20; n++)
    u -= 4. * pow(2. / pi, 3) * pow(-1., n) / pow(2 * n + 1., 3.) * cosh((2 * n + 1) * pi * x / 2.) *
         cos((2. * n + 1) * pi * y / 2.) / cosh((2 * n + 1) * pi * A / 2.);
  return u;
}

/* The inlet speed of profiles 2, 4, 7 and 10 (bcs.c:152-195) at face cell (i, j)
 * of the k = 0 face, from the mean of its four nodes (coor: the node
 * coordinates in the box layout [mz][my][mx][3]) less cm (CMx_c, CMy_c,
 * CMz_c). */
double orc_inlet_shaped(int inletprofile, const double *coor, int mx, int my, int i, int j, const double *cm) {
  const double *a = coor + 3 * ((size_t)j * mx + i), *b = coor + 3 * ((size_t)(j - 1) * mx + i);
  const double *c = coor + 3 * ((size_t)j * mx + i - 1), *d = coor + 3 * ((size_t)(j - 1) * mx + i - 1);
  const double xc = (a[0] + b[0] + c[0] + d[0]) * 0.25 - cm[0];
  const double yc = (a[1] + b[1] + c[1] + d[1]) * 0.25 - cm[1];
  const double zc = (a[2] + b[2] + c[2] + d[2]) * 0.25 - cm[2];
  const double r = sqrt(zc * zc + yc * yc);
  const double H = 4.1, Umax = 1.5;
  if (inletprofile == 2) return 4. * Umax * yc * (H - yc) / (H * H);
  if (inletprofile == 4) {
    double uin = 2. * (1. - 4. * r * r);
    if (r > 0.5) uin = 0.;
    return uin;
  }
  if (inletprofile == 10) return orc_duct_speed(xc, yc);
  if (inletprofile == 0) return table_speed(r);
  if (inletprofile == 5) return -table_speed(r);
  return 1.5 * (1. - 4. * yc * yc); /* 7 */
}

/* The inlet's nodes orc_inflow_flux and orc_imp_rk use for the shaped
 * profiles (the reference reads its coordinates and CMx_c, CMy_c, CMz_c as
 * globals too). */
static const double *g_inlet_coor;
static double g_inlet_cm[3];
void orc_set_inlet_nodes(const double *coor0, const double *cm) {
  g_inlet_coor = coor0;
  for (int d = 0; d < 3; d++) g_inlet_cm[d] = cm ? cm[d] : 0.;
}

static int inlet_covered(int inletprofile) {
  double uin;
  if (inletprofile == 2 || inletprofile == 4 || inletprofile == 7 || inletprofile == 10) return g_inlet_coor != NULL;
  if (inletprofile == 0 || inletprofile == 5) return g_inlet_coor != NULL && table_step_ok();
  return orc_inlet_speed(inletprofile, &uin);
}

int orc_inflow_flux(const orc_level *L, double *ucont, double *ub, int inletprofile, double *flux_in_sum) {
  return orc_inflow_flux_ext(L, ucont, ub, inletprofile, g_inlet_coor, g_inlet_cm, flux_in_sum);
}

int orc_inflow_flux_ext(const orc_level *L, double *ucont, double *ub, int inletprofile, const double *coor,
                        const double *cm, double *flux_in_sum) {
  const int mx = L->mx, my = L->my;
  if (L->bctype[4] != 5) return 0; /* FluxIn is 0 and FluxInSum keeps its value */
  double uin0 = 0.;
  const int shaped = inletprofile == 2 || inletprofile == 4 || inletprofile == 7 || inletprofile == 10 ||
                     inletprofile == 0 || inletprofile == 5;
  if ((inletprofile == 0 || inletprofile == 5) && !table_step_ok()) return -1;
  if (shaped ? !(coor && cm) : !orc_inlet_speed(inletprofile, &uin0)) return -1;
  const double *z;
  for (int j = 1; j < my - 1; j++)
    for (int i = 1; i < mx - 1; i++) {
      const size_t q = ID(L, i, j, 0);
      const double uin = shaped ? orc_inlet_shaped(inletprofile, coor, mx, my, i, j, cm) : uin0;
      if (!(L->nvert[ID(L, i, j, 1)] < 0.1)) continue;
      z = L->zet + 3 * q;
      ub[3 * q + 1] = uin * z[1] / sqrt(z[2] * z[2] + z[1] * z[1] + z[0] * z[0]);
      ub[3 * q + 2] = uin * z[2] / sqrt(z[2] * z[2] + z[1] * z[1] + z[0] * z[0]);
      ub[3 * q + 0] = uin * z[0] / sqrt(z[2] * z[2] + z[1] * z[1] + z[0] * z[0]);
      ucont[3 * q + 2] = uin * sqrt(z[2] * z[2] + z[1] * z[1] + z[0] * z[0]);
    }
  double f = 0;
  for (int j = 1; j < my - 1; j++)
    for (int i = 1; i < mx - 1; i++)
      if (L->nvert[ID(L, i, j, 1)] < 0.1) f += ucont[3 * ID(L, i, j, 0) + 2];
  *flux_in_sum = f;
  return 0;
}

/* One of FormBCS's edge averages: ucat and p at d become the means of their
 * values at a and b (bcs.c:5439-5570). */
static inline void edge_avg(double *u, double *p, long d, long a, long b) {
  avg3(u + 3 * d, u + 3 * a, u + 3 * b);
  p[d] = 0.5 * (p[a] + p[b]);
}

int orc_form_bcs(const orc_level *L, double *ucont, double *ub, double *u, double *p, double flux_in_sum,
                 double flux_intp_sum) {
  const int mx = L->mx, my = L->my, mz = L->mz;
  if (!orc_bcs_covered(L->bctype)) return -1;
#define U3(i, j, k) (u + 3 * ID(L, (i), (j), (k)))
#define B3(i, j, k) (ub + 3 * ID(L, (i), (j), (k)))
#define Q(i, j, k) ((long)ID(L, (i), (j), (k)))
  for (int pass = 0; pass < 3; pass++) { /* bcs.c:4483 */
    if (L->bctype[5] == 4) {             /* the outlet (bcs.c:4914-4998) */
      const int k = mz - 1;
      double flux_out = 0, area = 0;
      for (int j = 1; j < my - 1; j++)
        for (int i = 1; i < mx - 1; i++) {
          if (!(L->nvert[ID(L, i, j, k - 1)] < 0.1)) continue;
          const double *c = U3(i, j, k - 1), *z = L->zet + 3 * ID(L, i, j, k - 1);
          flux_out += (c[0] * z[0] + c[1] * z[1] + c[2] * z[2]);
          area += sqrt(z[0] * z[0] + z[1] * z[1] + z[2] * z[2]);
        }
      const double flux_in = flux_in_sum + 0. + flux_intp_sum; /* + FarFluxInSum, 0 here */
      const double ratio = (flux_in - flux_out) / area;
      for (int j = 1; j < my - 1; j++)
        for (int i = 1; i < mx - 1; i++) {
          if (!(L->nvert[ID(L, i, j, k - 1)] < 0.1)) continue;
          double *b = B3(i, j, k);
          const double *z = L->zet + 3 * ID(L, i, j, k - 1);
          copy3(b, U3(i, j, k - 1));
          ucont[3 * ID(L, i, j, k - 1) + 2] =
              (b[0] * z[0] + b[1] * z[1] + b[2] * z[2]) + ratio * sqrt(z[0] * z[0] + z[1] * z[1] + z[2] * z[2]);
        }
    }
    orc_contra2cart(L, ucont, u); /* bcs.c:5159 */
    /* ghost faces on the faces' interior cells (bcs.c:5250-5318) */
    for (int k = 1; k < mz - 1; k++)
      for (int j = 1; j < my - 1; j++) ghost3(U3(0, j, k), B3(0, j, k), U3(1, j, k));
    for (int k = 1; k < mz - 1; k++)
      for (int j = 1; j < my - 1; j++) ghost3(U3(mx - 1, j, k), B3(mx - 1, j, k), U3(mx - 2, j, k));
    for (int k = 1; k < mz - 1; k++)
      for (int i = 1; i < mx - 1; i++) ghost3(U3(i, 0, k), B3(i, 0, k), U3(i, 1, k));
    for (int k = 1; k < mz - 1; k++)
      for (int i = 1; i < mx - 1; i++) ghost3(U3(i, my - 1, k), B3(i, my - 1, k), U3(i, my - 2, k));
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) ghost3(U3(i, j, 0), B3(i, j, 0), U3(i, j, 1));
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) ghost3(U3(i, j, mz - 1), B3(i, j, mz - 1), U3(i, j, mz - 2));
    /* the 12 edges of ucat and p, in the reference's order (bcs.c:5439-5570) */
    for (int j = 0; j < my; j++) edge_avg(u, p, Q(0, j, 0), Q(0, j, 1), Q(1, j, 0));
    for (int j = 0; j < my; j++) edge_avg(u, p, Q(mx - 1, j, 0), Q(mx - 1, j, 1), Q(mx - 2, j, 0));
    for (int i = 0; i < mx; i++) edge_avg(u, p, Q(i, 0, 0), Q(i, 0, 1), Q(i, 1, 0));
    for (int i = 0; i < mx; i++) edge_avg(u, p, Q(i, my - 1, 0), Q(i, my - 1, 1), Q(i, my - 2, 0));
    for (int j = 0; j < my; j++) edge_avg(u, p, Q(0, j, mz - 1), Q(0, j, mz - 2), Q(1, j, mz - 1));
    for (int j = 0; j < my; j++) edge_avg(u, p, Q(mx - 1, j, mz - 1), Q(mx - 1, j, mz - 2), Q(mx - 2, j, mz - 1));
    for (int i = 0; i < mx; i++) edge_avg(u, p, Q(i, 0, mz - 1), Q(i, 0, mz - 2), Q(i, 1, mz - 1));
    for (int i = 0; i < mx; i++) edge_avg(u, p, Q(i, my - 1, mz - 1), Q(i, my - 1, mz - 2), Q(i, my - 2, mz - 1));
    for (int k = 0; k < mz; k++) edge_avg(u, p, Q(0, 0, k), Q(0, 1, k), Q(1, 0, k));
    for (int k = 0; k < mz; k++) edge_avg(u, p, Q(mx - 1, 0, k), Q(mx - 1, 1, k), Q(mx - 2, 0, k));
    for (int k = 0; k < mz; k++) edge_avg(u, p, Q(0, my - 1, k), Q(0, my - 2, k), Q(1, my - 1, k));
    for (int k = 0; k < mz; k++) edge_avg(u, p, Q(mx - 1, my - 1, k), Q(mx - 1, my - 2, k), Q(mx - 2, my - 1, k));
  }
#undef U3
#undef B3
#undef Q
  return 0;
}

/* VecNorm(NORM_INFINITY) as the PETSc shim computes it: the largest |x|. */
static double max_abs(const double *x, size_t n) {
  double s = 0;
  for (size_t q = 0; q < n; q++) {
    const double v = fabs(x[q]);
    s = v > s ? v : s;
  }
  return s;
}

int orc_imp_rk(const orc_level *L, double *ucont, const double *ucont_o, const double *ucont_rm1, double *ucat,
               double *p, double *ubcs, double ren, double dt, double st, double cfl, int ti, int tistart,
               int central, double atol, double rtol, int max_it, int inletprofile, double flux_intp_sum,
               orc_imp_rk_stats *out) {
  const size_t n3 = 3 * (size_t)L->mx * L->my * L->mz;
  const double alfa[4] = {0.25, 1 / 3., 0.5, 1.}; /* implicitsolver.c:7111 */
  double flux_in_sum = 0.;
  g_ti = ti; /* InletInterpolation reads the global ti */
  if (!orc_bcs_covered(L->bctype) || (L->bctype[4] == 5 && !inlet_covered(inletprofile))) return -1;
  /* InflowFlux, OutflowFlux (only sums what nothing here reads), FormBCS */
  orc_inflow_flux(L, ucont, ubcs, inletprofile, &flux_in_sum);
  orc_form_bcs(L, ucont, ubcs, ucat, p, flux_in_sum, flux_intp_sum);
  double *rhs = (double *)calloc(n3, sizeof(double)), *pu = (double *)malloc(sizeof(double) * n3);
  memcpy(pu, ucont, sizeof(double) * n3);
  orc_calc_rhs(L, ucont, ucont_o, ucont_rm1, ucat, p, ren, dt, ti, tistart, central, rhs);
  double normF0 = max_abs(rhs, n3), normF1 = 1000., normdU1 = 1000., lambda = cfl;
  double normdU = 10., reldU = 1., normdU_bk = 0., reldU_bk = 1., normdU0 = 0., normF_bk = 0., relF_bk = 0.;
  int pseudot = 0, rejected = 0;
  /* implicitsolver.c:7149-7239 */
  while (((normdU > atol && reldU > rtol) || pseudot < 1) && pseudot < max_it) {
    pseudot++;
    for (int s = 0; s < 4; s++) {
      const double a = lambda * alfa[s] * dt * st;
      for (size_t q = 0; q < n3; q++) ucont[q] = a * rhs[q] + pu[q];
      orc_inflow_flux(L, ucont, ubcs, inletprofile, &flux_in_sum);
      orc_form_bcs(L, ucont, ubcs, ucat, p, flux_in_sum, flux_intp_sum);
      orc_calc_rhs(L, ucont, ucont_o, ucont_rm1, ucat, p, ren, dt, ti, tistart, central, rhs);
    }
    normdU1 = normdU_bk;
    normdU_bk = 0;
    for (size_t q = 0; q < n3; q++) {
      const double v = fabs(-1. * ucont[q] + pu[q]);
      normdU_bk = v > normdU_bk ? v : normdU_bk;
    }
    if (pseudot == 1) {
      normdU0 = normdU_bk;
      reldU_bk = 1.;
    } else if (normdU0 > 1.e-10)
      reldU_bk = normdU_bk / normdU0;
    if (pseudot > 1) normF1 = normF_bk;
    normF_bk = max_abs(rhs, n3);
    if (pseudot == 1) normF0 = normF_bk;
    relF_bk = normF_bk / normF0;
    normdU = normdU_bk;
    reldU = reldU_bk;
    if (pseudot > 1 && normF_bk > normF1 && normdU_bk > normdU1 && lambda > 0.001) {
      lambda = 0.5 * lambda;
      pseudot--;
      rejected++;
      memcpy(ucont, pu, sizeof(double) * n3);
    } else {
      memcpy(pu, ucont, sizeof(double) * n3);
      normF1 = normF_bk;
      normdU1 = normdU_bk;
    }
  }
  free(rhs);
  free(pu);
  if (out) {
    out->pseudo_iterations = pseudot;
    out->rejected = rejected;
    out->norm_du = normdU;
    out->rel_du = reldU;
    out->norm_f = normF_bk;
    out->rel_f = relF_bk;
    out->lambda = lambda;
  }
  return 0;
}
