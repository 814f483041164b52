// The immersed-body classification of ibm_search_advanced (ibm.c:4197-4740):
// which cells of the finest level lie inside a closed triangle mesh, and the
// layer of cells around them.  FP64 with every operation rounded on its own,
// in the reference's order, so that every inside/outside decision, and with it
// nvert, equals the reference's bit for bit.
#include "cvb_internal.h"

namespace cvb {

static inline unsigned nblk(size_t n, int t) { return (unsigned)((n + t - 1) / t); }

__device__ __forceinline__ double im_(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ia_(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double is_(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double idot(const double *a, const double *b) {
  return ia_(ia_(im_(a[0], b[0]), im_(a[1], b[1])), im_(a[2], b[2]));
}

// intsect_triangle (compgeom.c:17-50): the ray o + t d against the triangle
// (v0, v0 + e1, v0 + e2); 1 with t on a hit.  The edges e1 = v1 - v0 and
// e2 = v2 - v0 come precomputed (the same IEEE subtractions).  The test u < 0,
// with u = (tv . pv) * (1 / det), is decided from the signs before dividing when
// the product cannot underflow to -0 (|tv . pv| >= 2^-1000, |det| <= 2^20):
// a nonzero product has the sign of its factors, so the decision is the
// reference's.  Everything else is computed as the reference computes it.
__device__ __forceinline__ int ray_hits(const double *o, const double *d, const double *v0, const double *e1,
                                        const double *e2, double *t) {
  double pv[3], tv[3], qv[3];
  pv[0] = is_(im_(d[1], e2[2]), im_(d[2], e2[1]));
  pv[1] = is_(im_(d[2], e2[0]), im_(d[0], e2[2]));
  pv[2] = is_(im_(d[0], e2[1]), im_(d[1], e2[0]));
  const double det = idot(e1, pv);
  if (det > -0.00000001 && det < 0.00000001) return 0;
#pragma unroll
  for (int c = 0; c < 3; c++) tv[c] = is_(o[c], v0[c]);
  const double nu = idot(tv, pv);
  if (fabs(nu) >= 0x1p-1000 && fabs(det) <= 0x1p20 && ((nu < 0.0) != (det < 0.0))) return 0;
  const double inv = __ddiv_rn(1.0, det);
  const double u = im_(nu, inv);
  if (u < 0.0 || u > 1.0) return 0;
  qv[0] = is_(im_(tv[1], e1[2]), im_(tv[2], e1[1]));
  qv[1] = is_(im_(tv[2], e1[0]), im_(tv[0], e1[2]));
  qv[2] = is_(im_(tv[0], e1[1]), im_(tv[1], e1[0]));
  const double v = im_(idot(d, qv), inv);
  if (v < 0.0 || ia_(u, v) > 1.0) return 0;
  *t = im_(idot(e2, qv), inv);
  return 1;
}

// point_cell_advanced (ibm.c:1285-1400) with randomdirection (ibm.c:87-118):
// a ray from p toward a point above the body's bounding box, aimed into the
// bucket column (ic, kc) with offset s[seed], crosses the column's triangles an
// odd number of times when p is inside.  A ray that meets two hits at the same
// distance on faces not facing apart (an edge or a vertex) is singular, and the
// next seed's ray is tried.  Returns 4 (inside), 0 (outside), or -1 when every
// one of the IbmArgs::tries rays was singular, or a ray met more than
// kIbmMaxHits faces.
__device__ int ibm_point_inside(const IbmArgs &A, const double *p, int ic, int jc, int kc) {
  double dt[kIbmMaxHits], dn[kIbmMaxHits][3];
  const int col = kc * kIbmBuckets + ic;
  const int q0 = A.col_start[col], q1 = A.col_start[col + 1];
  const double xpc = ia_(im_(A.dc[0], (double)ic + 0.5), A.min[0]);
  const double zpc = ia_(im_(A.dc[2], (double)kc + 0.5), A.min[2]);
  for (int seed = 1; seed <= A.tries; seed++) {
    const double s = A.offsets[seed - 1];
    double d[3];
    d[0] = is_(ia_(xpc, im_(s, A.dc[0])), p[0]);
    d[1] = is_(ia_(A.max[1], 0.2), p[1]);
    d[2] = is_(ia_(zpc, im_(s, A.dc[2])), p[2]);
    const double len = __dsqrt_rn(idot(d, d));
    d[0] = __ddiv_rn(d[0], len);
    d[1] = __ddiv_rn(d[1], len);
    d[2] = __ddiv_rn(d[2], len);
    int hits = 0;
    bool singular = false;
    for (int q = q0; q < q1 && !singular; q++) {
      const int2 ent = A.col_ent[q];  // (triangle, end of its bucket range in j)
      if (ent.y <= jc) continue;
      const double *T = A.tri + 12 * (size_t)ent.x;  // v0, e1, e2, unit normal
      double t;
      if (!ray_hits(p, d, T, T + 3, T + 6, &t)) continue;
      if (!(t > 0)) continue;
      const double *n = T + 9;
      if (hits == kIbmMaxHits) return -1;
      for (int h = 0; h < hits; h++)
        if (fabs(is_(t, dt[h])) < 1.e-8 && idot(dn[h], n) > -0.97) singular = true;
      dt[hits] = t;
      dn[hits][0] = n[0]; dn[hits][1] = n[1]; dn[hits][2] = n[2];
      hits++;
    }
    if (!singular) return (hits & 1) ? 4 : 0;
  }
  return -1;
}

// The inside test on the interior cells (ibm.c:4337-4357) in three passes, so
// that the ray casts run column by column: a warp then takes cells of one
// bucket column, which walk the same triangle list with nearly the same rays.
// 1. Every interior cell: the reset of body 0, the bounding-box test, and a
//    count of the cells in each bucket column.
__global__ void __launch_bounds__(256) k_ibm_select(IbmArgs A, int *key, int *count) {
  const Geom &g = A.g;
  const int ni = g.mx - 2, nj = g.my - 2;
  const size_t cells = (size_t)ni * nj * (g.mz - 2);
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= cells) return;
  const int i = 1 + (int)(t % ni), j = 1 + (int)((t / ni) % nj), k = 1 + (int)(t / ((size_t)ni * nj));
  const size_t q = ((size_t)k * g.my + j) * g.mx + i;
  double nv = A.nvert[q];
  if (A.ibi == 0 && nv < 5.) {
    nv = 0;
    A.nvert[q] = nv;
  }
  const double *c = A.cent + 3 * q;
  int col = -1;
  if (c[0] > A.min[0] && c[0] < A.max[0] && c[1] > A.min[1] && c[1] < A.max[1] && c[2] > A.min[2] &&
      c[2] < A.max[2]) {
    const int ic = (int)floor(__ddiv_rn(is_(c[0], A.min[0]), A.dc[0]));
    const int kc = (int)floor(__ddiv_rn(is_(c[2], A.min[2]), A.dc[2]));
    col = kc * kIbmBuckets + ic;
    atomicAdd(count + col, 1);
  }
  key[t] = col;
}

// 2. Start of each column's run in the cell list (exclusive scan of the counts;
//    one block, kIbmBuckets^2 columns).  fill[] is zeroed for pass 3.
__global__ void __launch_bounds__(1024) k_ibm_scan(const int *count, int *start, int *fill) {
  constexpr int ncol = kIbmBuckets * kIbmBuckets, per = (ncol + 1023) / 1024;
  __shared__ int part[1024];
  const int t = threadIdx.x;
  int local = 0;
  for (int u = 0; u < per; u++) {
    const int c = t * per + u;
    if (c < ncol) local += count[c];
  }
  part[t] = local;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {  // inclusive scan of the per-thread sums
    const int v = t >= o ? part[t - o] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  int run = part[t] - local;
  for (int u = 0; u < per; u++) {
    const int c = t * per + u;
    if (c < ncol) {
      start[c] = run;
      fill[c] = 0;
      run += count[c];
    }
  }
}

// 3. Each selected cell takes a slot in its column's run.
__global__ void __launch_bounds__(256) k_ibm_scatter(Geom g, const int *key, const int *start, int *fill, int *list) {
  const size_t cells = (size_t)(g.mx - 2) * (g.my - 2) * (g.mz - 2);
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= cells) return;
  const int col = key[t];
  if (col >= 0) list[start[col] + atomicAdd(fill + col, 1)] = (int)t;
}

__global__ void k_ibm_total(const int *start, const int *count, int *total) {
  constexpr int last = kIbmBuckets * kIbmBuckets - 1;
  *total = start[last] + count[last];
}

// 4. The ray cast of every listed cell (interior-cell number t).
__global__ void __launch_bounds__(128) k_ibm_inside(IbmArgs A, const int *list, const int *nlisted) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= *nlisted) return;
  const Geom &g = A.g;
  const int ni = g.mx - 2, nj = g.my - 2;
  const size_t t = (size_t)list[s];
  const int i = 1 + (int)(t % ni), j = 1 + (int)((t / ni) % nj), k = 1 + (int)(t / ((size_t)ni * nj));
  const size_t q = ((size_t)k * g.my + j) * g.mx + i;
  const double *c = A.cent + 3 * q;
  const int ic = (int)floor(__ddiv_rn(is_(c[0], A.min[0]), A.dc[0]));
  const int jc = (int)floor(__ddiv_rn(is_(c[1], A.min[1]), A.dc[1]));
  const int kc = (int)floor(__ddiv_rn(is_(c[2], A.min[2]), A.dc[2]));
  const int r = ibm_point_inside(A, c, ic, jc, kc);
  if (r < 0) {
    atomicOr(A.failed, 1);
    return;
  }
  double nv = A.nvert[q];
  if (nv < r) nv = r;
  if (nv < 0) nv = 0;
  A.nvert[q] = nv;
}

// The layer around inside cells (ibm.c:4415-4437), every cell of the box, from
// src into dst.  The reference updates in place, but no cell becomes inside
// (4) there, so every cell's test sees the same inside cells either way.  The
// inside cells are marked first, one byte a cell: the test (int)(nv + 0.5) == 4
// then runs once per cell instead of 27 times (both its operations run on the
// FP64 pipe).
__global__ void k_ibm_mark(Geom g, const double *__restrict__ nv, unsigned char *__restrict__ in4) {
  const size_t n = g.n(), q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) in4[q] = (int)(nv[q] + 0.5) == 4;
}
__global__ void k_ibm_layer(Geom g, const double *__restrict__ src, const unsigned char *__restrict__ in4,
                            double *__restrict__ dst) {
  const size_t n = g.n(), q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int i = (int)(q % g.mx), j = (int)((q / g.mx) % g.my), k = (int)(q / ((size_t)g.mx * g.my));
  double nv = src[q];
  if (nv < 0) nv = 0;
  if (!in4[q]) {
    const int ip = i < g.mx - 1 ? i + 1 : i, im = i > 0 ? i - 1 : i;
    const int jp = j < g.my - 1 ? j + 1 : j, jm = j > 0 ? j - 1 : j;
    const int kp = k < g.mz - 1 ? k + 1 : k, km = k > 0 ? k - 1 : k;
    int near = 0;
    for (int kk = km; kk <= kp; kk++)
      for (int jj = jm; jj <= jp; jj++)
        for (int ii = im; ii <= ip; ii++) near |= in4[((size_t)kk * g.my + jj) * g.mx + ii];
    if (near) nv = 2 < nv ? nv : 2;
  }
  dst[q] = nv;
}

// The phase-change fix against the previous step's nvert (ibm.c:4499-4509,
// after the last body) and this body's codes 1 / 3 + ibi/1000 (ibm.c:4651-4659).
// Each cell's class for the clean-up, (int)nv: 0 (fluid), 1 (IB) or other (2),
// goes into a byte.
__global__ void k_ibm_codes(Geom g, double *nvert, const double *__restrict__ nvert_o, int ibi, int last,
                            unsigned char *__restrict__ cls) {
  const size_t n = g.n(), q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  double nv = nvert[q];
  if (last && nvert_o[q] > 2.5 && nv < 0.5) nv = 2;
  if ((int)(nv + 0.5) == 2) nv = ia_(1.0, __ddiv_rn((double)ibi, 1000.0));
  if ((int)(nv + 0.5) == 4) nv = ia_(3.0, __ddiv_rn((double)ibi, 1000.0));
  nvert[q] = nv;
  const int c = (int)nv;
  cls[q] = c == 0 ? 0 : c == 1 ? 1 : 2;
}

// Two clean-up passes (ibm.c:4662-4690): an IB cell ((int)nv == 1, so nv in
// [1, 2)) whose k neighbours are both fluid ((int)nv == 0) becomes
// min(0, nv) = 0.  The reference sweeps k upward in place, so a cell sees the
// new value below it and the old one above: one thread walks each interior
// (i, j) column in that order, on the class bytes.
__global__ void k_ibm_around(Geom g, double *nvert, unsigned char *cls) {
  const int ni = g.mx - 2, nj = g.my - 2;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ni * nj) return;
  const int i = 1 + t % ni, j = 1 + t / ni;
  const size_t plane = (size_t)g.mx * g.my, c = (size_t)j * g.mx + i;
  for (int pass = 0; pass < 2; pass++) {
    int below = cls[c], cur = cls[plane + c];
    for (int k = 1; k < g.mz - 1; k++) {
      const size_t q = k * plane + c;
      const int above = cls[q + plane];
      if (cur == 1 && below == 0 && above == 0) {
        cur = 0;
        cls[q] = 0;
        nvert[q] = 0;
      }
      below = cur;
      cur = above;
    }
  }
}

void launch_ibm_search(const IbmArgs &A, const IbmWork &W, double *tmp, cudaStream_t s) {
  const Geom &g = A.g;
  const size_t inner = (size_t)(g.mx - 2) * (g.my - 2) * (g.mz - 2), n = g.n();
  if (inner) {
    constexpr int ncol = kIbmBuckets * kIbmBuckets;
    cudaMemsetAsync(W.count, 0, sizeof(int) * ncol, s);
    k_ibm_select<<<nblk(inner, 256), 256, 0, s>>>(A, W.key, W.count);
    count_launch();
    k_ibm_scan<<<1, 1024, 0, s>>>(W.count, W.start, W.fill);
    count_launch();
    k_ibm_scatter<<<nblk(inner, 256), 256, 0, s>>>(g, W.key, W.start, W.fill, W.list);
    count_launch();
    // the number of listed cells is the last column's start + count; read on
    // the device, so the grid covers every interior cell and threads past it return
    k_ibm_total<<<1, 1, 0, s>>>(W.start, W.count, W.total);
    count_launch();
    k_ibm_inside<<<nblk(inner, 128), 128, 0, s>>>(A, W.list, W.total);
    count_launch();
  }
  k_ibm_mark<<<nblk(n, 256), 256, 0, s>>>(g, A.nvert, W.in4);
  count_launch();
  k_ibm_layer<<<nblk(n, 256), 256, 0, s>>>(g, A.nvert, W.in4, tmp);
  count_launch();
  // the layer is done with the inside marks: their bytes take the classes
  k_ibm_codes<<<nblk(n, 256), 256, 0, s>>>(g, tmp, A.nvert_o, A.ibi, A.ibi == A.nbodies - 1, W.in4);
  count_launch();
  k_ibm_around<<<nblk((size_t)(g.mx - 2) * (g.my - 2), 128), 128, 0, s>>>(g, tmp, W.in4);
  count_launch();
}

}  // namespace cvb
