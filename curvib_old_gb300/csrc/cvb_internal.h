// Internal declarations shared by the CUDA kernels and the host library.
// Grid layout everywhere: one level is the reference's DMDA box [mz][my][mx],
// i fastest, boundary ring included (mx = IM+1 for IM nodes).
#pragma once
#include <functional>
#include <cuda_runtime.h>
#include <stdint.h>

namespace cvb {

// Kernel launches issued by this library (all contexts), for measurement.
void count_launch(int n = 1);
long long launch_count();

// Stencil slots, in the order of the reference's PoissonLHSNew (poisson.c:576-594).
enum Slot { CP, EP, WP, NP, SP, TP, BP, NE, SE, NW, SW, TN, BN, TS, BS, TE, BE, TW, BW, NSLOT };

// Per-cell switching code (built once from nvert by build_codes):
//   bit 0       identity row (boundary ring, or nvert > 0.1)
//   bits 1..6   face active from this row's side: E, W, N, S, T, B
//   bit 7       blocked: nvert > 0.1 (read by the grid transfers)
//   bit 20      fluid: interior and nvert < 0.1
//   bits 8..19  cross-derivative form for this cell's three upper faces, 2 bits each:
//               E: (j, k)  N: (i, k)  T: (i, j)   0 none, 1 central, 2 lower, 3 upper
// A lower face (W/S/B) of a row is the upper face of its lower neighbour, so a
// row reads that neighbour's code for it.
enum : uint32_t {
  CODE_IDENTITY = 1u,
  CODE_BLOCKED = 1u << 7,  // nvert > 0.1 (IB or solid), any cell
  CODE_FLUID = 1u << 20,   // interior cell with nvert < 0.1 (the null space's and range projection's cells)
  CODE_ACT_E = 1u << 1, CODE_ACT_W = 1u << 2, CODE_ACT_N = 1u << 3,
  CODE_ACT_S = 1u << 4, CODE_ACT_T = 1u << 5, CODE_ACT_B = 1u << 6,
};
__host__ __device__ inline int code_branch(uint32_t c, int face, int which) {
  return (c >> (8 + 4 * face + 2 * which)) & 3u;  // face 0=E,1=N,2=T; which 0/1
}

struct Geom {
  int mx, my, mz;
  int px, py, pz;  // periodic directions (bctype 7)
  __host__ __device__ size_t n() const { return (size_t)mx * my * mz; }
  __host__ __device__ size_t id(int i, int j, int k) const {
    return ((size_t)k * my + j) * mx + i;
  }
  // neighbour index with the reference's periodic wrap of column indices
  __host__ __device__ int iu(int i) const { return (px && i == mx - 2) ? 1 : i + 1; }
  __host__ __device__ int id_(int i) const { return (px && i == 1) ? mx - 2 : i - 1; }
  __host__ __device__ int ju(int j) const { return (py && j == my - 2) ? 1 : j + 1; }
  __host__ __device__ int jd(int j) const { return (py && j == 1) ? my - 2 : j - 1; }
  __host__ __device__ int ku(int k) const { return (pz && k == mz - 2) ? 1 : k + 1; }
  __host__ __device__ int kd(int k) const { return (pz && k == 1) ? mz - 2 : k - 1; }
};

// Thomas factors in global memory, line by line: line (i, k) holds a_j, 1/m_j
// and c'_j for j = 1..my-2 as three runs of Q = my-2 rounded up to 4 values
// (zero-padded), so that a line's factors are 16-byte aligned and contiguous.
// Lines are ordered by plane k, then zebra colour (i + k) % 2, then i / 2: the
// lines of one colour in one plane -- the tile of a zebra line solve -- follow
// one another.
struct LineFac {
  int nt, Q;
  __host__ __device__ static LineFac of(const Geom &g) {
    LineFac f;
    f.nt = (g.mx + 1) >> 1;
    f.Q = (g.my - 2 + 3) & ~3;
    return f;
  }
  __host__ __device__ size_t line(int i, int k) const {
    return (((size_t)k * 2 + ((i + k) & 1)) * nt + (i >> 1)) * 3 * (size_t)Q;
  }
  __host__ __device__ size_t count(const Geom &g) const { return (size_t)g.mz * 2 * nt * 3 * Q; }
};

// Colour-split rows: the cells of zebra colour (i + k) % 2 == c of row (j, k)
// at c * half + i / 2 of a row of 2 * half slots.  A zebra half-sweep passes
// its residual to the line solves in this layout, so that the lines of one
// colour are adjacent in memory.
struct SplitRow {
  __host__ __device__ static int half(const Geom &g) { return (g.mx + 1) >> 1; }
  __host__ __device__ static size_t count(const Geom &g) { return (size_t)g.my * g.mz * 2 * half(g); }
  __host__ __device__ static int at(const Geom &g, int i, int j, int k) {
    const int h = half(g);
    return (k * g.my + j) * 2 * h + ((i + k) & 1) * h + (i >> 1);
  }
};

// Device data of one multigrid level.
struct LevelDev {
  Geom g;
  int isc, jsc, ksc;     // semi-coarsening flags of this level (GridRestriction)
  double *nvert;         // [N]
  uint32_t *code;        // [N]
  double *w64;           // [19][N] FP64 stencil weights (rows scaled by -aj; identity rows CP=1)
  float *gf32;           // [9][N]  FP32 face coefficients g11..g33, cross terms pre-scaled by form weight
  float *ajf32;          // [N]
  float *wgt32;          // [N]    restriction weight max(0, 1 - nvert), rounded to float
  float *line32;         // y-line Thomas factors (a_j, 1/m_j, c'_j) in FP32, LineFac layout
  float *cs32;           // levels without FP32 cross terms: g11, g22, g33, aj and the code (its bits)
                         // in colour-split rows ([5][SplitRow::count]) for the zebra residual; else null
  double *line64;        // ... in FP64
  // work vectors of this level (the finest level's b/x live in the solver)
  double *r64, *e64, *t64;  // FP64 V-cycle vectors
  float *r32, *e32, *t32;   // FP32 V-cycle vectors
  int sweep32, sweep64;     // line-sweep variant chosen at set-up: 0 fused, 1 split
  // the operator has cross-derivative terms (FP32 flux form / FP64 edge
  // weights); 0 on an orthogonal grid, where the kernels read 7 points
  int cross32, cross64;
  int zfuse32, zfuse64;     // zebra variant chosen at set-up: 0 two kernels per half-sweep, 1 one
                            // (in place without cross terms, else out of place)
  int ztma32;               // FP32 zebra half-sweep with TMA-staged tiles (kernels_tma.cu): the
                            // row pairs per chunk (4, 8, 16) the autotuner chose, 0 off
  int ztw32;                // lines per block of the FP32 zebra line-solve tiles (4 or 8; 0: 8)
  // coarsest level only: the densely inverted cells (first cm of cidx) and the
  // identity ones (the rest of cidx)
  const int *cidx;
  int cm;
  // When set, every kernel launched for this level returns at once while *gate
  // is non-zero: an FGMRES iteration issued ahead of the host's convergence
  // check turns into no-ops once the previous iteration has converged.
  const int *gate;
};

__device__ __forceinline__ bool gated(const int *gate) { return gate && *gate; }

// Whether a level's operator in precision T has cross-derivative terms.
template <typename T>
__host__ __device__ inline bool has_cross(const LevelDev &L) {
  return sizeof(T) == 4 ? L.cross32 != 0 : L.cross64 != 0;
}

// The fused zebra half-sweep's condition (see zebra_fused_body): no
// cross-derivative terms, and colours kept apart across periodic seams.
template <typename T>
__host__ __device__ inline bool zebra_fusable(const LevelDev &L) {
  return !has_cross<T>(L) && (!L.g.px || (L.g.mx & 1) == 0) && (!L.g.pz || (L.g.mz & 1) == 0);
}


// --- kernel launchers (defined in the .cu files) ---------------------------
// setup
void launch_gcoef(const Geom &g, const double *const *metric /*12 Cmpnts fields: I(csi,eta,zet) J.. K..*/,
                  const double *iaj, const double *jaj, const double *kaj, double *g9 /*[9][N]*/,
                  cudaStream_t s);
void launch_codes(const Geom &g, const double *nvert, uint32_t *code, cudaStream_t s);
// wgt32 = (float) max(0, 1 - nvert)
void launch_weight32(const Geom &g, const double *nvert, float *wgt32, cudaStream_t s);
// flags[0] |= some FP32 cross coefficient is non-zero, flags[1] |= some FP64
// edge weight is non-zero (flags zeroed by the caller)
void launch_cross_flags(const Geom &g, const float *gf32, const double *w64, int *flags, cudaStream_t s);
// FP32 face coefficients: cross terms pre-scaled by their form's weight (after launch_codes)
void launch_scale_cross(const Geom &g, const uint32_t *code, float *gf32, cudaStream_t s);
void launch_weights(const Geom &g, const double *g9, const double *aj, const double *nvert,
                    const uint32_t *code, double *w64, cudaStream_t s);
void launch_line_factors(const Geom &g, const double *w64, double *line64, float *line32,
                         cudaStream_t s);
void launch_to_f32(const double *a, float *b, size_t n, cudaStream_t s, const int *gate = nullptr);
void launch_nvert_restrict(const Geom &fine, const double *nvf, const Geom &coarse, int isc, int jsc,
                           int ksc, double *nvc, double *tmp, cudaStream_t s);

// operator / smoother / transfers (T = float or double)
template <typename T>
void launch_apply(const LevelDev &L, const T *x, T *y, cudaStream_t s);
template <typename T>
void launch_residual(const LevelDev &L, const T *b, const T *x, T *r, cudaStream_t s);
template <typename T>
void launch_line_smooth(const LevelDev &L, const T *b, const T *x, T *xnew, T omega, int zero_guess,
                        cudaStream_t s);
// The FP32 zebra half-sweep of one colour in place with TMA-staged tiles of
// rp row pairs (kernels_tma.cu); false when the level does not allow it.
bool zebra_tma_ok(const LevelDev &L);
bool launch_zebra_tma(const LevelDev &L, const float *b, float *x, float omega, int color, int rp, cudaStream_t s);
// 1 if a TMA kernel's bounded wait gave up since the last call (cleared), 0 if
// not, -1 on a CUDA error; synchronises the stream.
int tma_timeout_take(cudaStream_t s);
// zebra half-sweep of one color, in place (res: scratch for the residual)
template <typename T>
void launch_zebra_half(const LevelDev &L, const T *b, T *x, T *res, T omega, int color, bool zero, cudaStream_t s);
// one zebra sweep (both colours) on x; tmp: a level-sized buffer for the
// out-of-place one-kernel form; zero_first: x is zero on entry
template <typename T>
void launch_zebra_sweep(const LevelDev &L, const T *b, T *x, T *tmp, T *res, T omega, bool zero_first, cudaStream_t s);
// restriction of xf into xc; zero_c, when set, is zeroed over the coarse grid too
template <typename T>
void launch_restrict(const LevelDev &F, const LevelDev &C, const T *xf, T *xc, cudaStream_t s, T *zero_c = nullptr);
template <typename T>
void launch_prolong_add(const LevelDev &C, const LevelDev &F, const T *xc, T *xf, cudaStream_t s);

// mixed-precision glue: FP64 operator on an FP32-stored vector
void launch_apply64_from32(const LevelDev &L, const float *x, double *y, cudaStream_t s);
void launch_f64_to_f32(const double *a, float *b, size_t n, cudaStream_t s, const int *gate = nullptr);
void launch_f32_to_f64(const float *a, double *b, size_t n, cudaStream_t s, const int *gate = nullptr);

// Krylov support (deterministic two-stage reductions)
int reduce_blocks();
int sm_count();
void launch_multidot(const double *const *V, int nv, const double *w, size_t n, double *partial,
                     cudaStream_t s, int self = 0, const int *gate = nullptr);
void launch_multidot_f32(const float *const *V, int nv, const double *w, size_t n, double *partial,
                         cudaStream_t s);
void launch_finish_sums(const double *partial, int nv, int nblocks, double *out, cudaStream_t s,
                        const int *gate = nullptr);
void launch_multiaxpy_norm(double *w, const double *const *V, const double *h_dev, int nv, size_t n,
                           double *partial, cudaStream_t s, const int *gate = nullptr);
// dst = src / *scal_dev (and, with dst32, its FP32 copy)
void launch_scale(double *dst, const double *src, const double *scal_dev, size_t n, cudaStream_t s,
                  const int *gate = nullptr, float *dst32 = nullptr);
// dst = src / sqrt(*sq_dev) (and, with dst32, its FP32 copy)
void launch_scale_sqrt(double *dst, const double *src, const double *sq_dev, size_t n, cudaStream_t s,
                       float *dst32 = nullptr, const int *gate = nullptr);
// cs[5][SplitRow::count] = g11, g22, g33 (gf32 slots 0, 4, 8), aj and the code's
// bits, each cell at its colour-split position
void launch_split_coef(const Geom &g, const float *gf32, const float *ajf32, const uint32_t *code, float *cs,
                       cudaStream_t s);
// out = 1 / a, element by element (correctly rounded)
void launch_reciprocal(const double *a, double *out, size_t n, cudaStream_t s);
void launch_axpy_z(double *x, const float *const *Z32, const double *const *Z64, const double *y_dev,
                   int nz, size_t n, cudaStream_t s);
void launch_fluid_mean_partial(const Geom &g, const uint32_t *code, const double *x, double *partial,
                               cudaStream_t s);
void launch_add_fluid_const(const Geom &g, const uint32_t *code, double *x, const double *sumcnt,
                            int zero_outside, cudaStream_t s);
// range projection of a right-hand side: sums of b/aj (b times the stored 1/aj)
// and counts over fluid cells, then b -= aj * sum/count there
void launch_fluid_ratio_partial(const Geom &g, const uint32_t *code, const double *b, const double *inv_aj,
                                double *partial, cudaStream_t s);
void launch_remove_aj_mean(const Geom &g, const uint32_t *code, const double *aj, double *b, const double *sums,
                           cudaStream_t s);
// b / a for the range projection's sum: an FP32 reciprocal refined by two
// Newton-Raphson steps in FP64 (r <- r + r (1 - a r)), within a unit or so in
// the last place of the quotient, at a fraction of an FP64 division's cost on
// this part (whose FP64 rate is low); a plain division where the FP32
// reciprocal cannot represent 1/a.
__device__ __forceinline__ double quot_newton(double b, double a) {
  const float af = (float)a;
  double r = (double)__frcp_rn(af);
  if (!(r != 0.0 && r * 0.0 == 0.0)) return b / a;
  r = fma(r, fma(-a, r, 1.0), r);
  r = fma(r, fma(-a, r, 1.0), r);
  return b * r;
}
// coarsest solve e = M^-1 r on C.cidx[0..C.cm), e = r on the other cells
// In-place Gauss-Jordan inverse of the n x n row-major A on the device into
// out (kernels_setup.cu); false for a singular matrix.  Work arrays: perm and
// colmap n ints, prow and fcol n doubles, status one int.
bool device_dense_inverse(double *A, int n, double *out, int *perm, int *colmap, double *prow, double *fcol,
                          int *status, cudaStream_t s);
void launch_dense_apply(const LevelDev &C, const double *Minv, const double *r, double *e, cudaStream_t s,
                        const int *gate = nullptr);
void launch_dense_apply_f32(const LevelDev &C, const double *Minv, const float *r, float *e, cudaStream_t s,
                            const int *gate = nullptr);

// projection-path kernels (FP64)
void launch_poisson_rhs(const Geom &g, const double *ucont, const double *aj, const double *nvert,
                        double dt, double st, double *b, double *partial, cudaStream_t s);
void launch_ib_sums(const Geom &g, const double *ucont, const double *csi, const double *eta,
                    const double *zet, const double *nvert, double *partial, cudaStream_t s);
void launch_ib_correct(const Geom &g, double *ucont, const double *csi, const double *eta,
                       const double *zet, const double *nvert, const double *flux_area,
                       double flux_intp_sum, int flg, cudaStream_t s);
void launch_update_pressure(const Geom &g, double *p, double *phi, cudaStream_t s);
void launch_projection(const Geom &g, const double *const *fm /*I,J,K csi/eta/zet*/, const double *iaj,
                       const double *jaj, const double *kaj, const double *nvert, const double *phi,
                       double dt, double st, double *ucont, cudaStream_t s);
// Immersed-body classification (kernels_ibm.cu).  The body's bounding box is
// cut into kIbmBuckets^3 buckets (ibm.c:4213); a ray from a cell centre walks
// one bucket column upward.
constexpr int kIbmBuckets = 40, kIbmMaxHits = 32, kIbmMaxTries = 64;
struct IbmArgs {
  Geom g;
  double min[3], max[3], dc[3];  // bounding box and bucket size
  const int *col_start;          // bucket column (i, k) = k * kIbmBuckets + i -> its entries
  const int2 *col_ent;           // (triangle, end of the triangle's bucket range in j)
  const double *tri;             // per triangle: v0, v1 - v0, v2 - v0, unit normal (12 doubles)
  const double *offsets;         // ray offset of seeds 1 .. tries (randomdirection's s)
  int tries;
  const double *cent;            // cell centres, [mz][my][mx][3]
  double *nvert;                 // [mz][my][mx], updated in place
  const double *nvert_o;         // the previous step's nvert
  int ibi, nbodies;
  int *failed;                   // set when a cell found no usable ray
};
// Work arrays of the search: per interior cell its bucket column (key) and
// the cell list sorted by column (list); per column its count, start and fill;
// per cell of the box a byte marking inside cells (in4).
struct IbmWork {
  int *key, *list, *count, *start, *fill, *total;
  unsigned char *in4;
};
// The search; tmp is one more [mz][my][mx] array.  The result is left in tmp.
void launch_ibm_search(const IbmArgs &A, const IbmWork &W, double *tmp, cudaStream_t s);

// fac: the grid's Contra2Cart factors (launch_c2c_factors, 10 N doubles), or
// null to form them in the kernel
void launch_contra2cart(const Geom &g, const double *csi, const double *eta, const double *zet,
                        const double *nvert, const double *ucont, double *ucat, cudaStream_t s, int k0 = 1,
                        int nk = -1, const double *fac = nullptr);
void launch_c2c_factors(const Geom &g, const double *csi, const double *eta, const double *zet, double *fac,
                        cudaStream_t s);
// max |div| and its first box index into out_v / out_i (device); pv / pi
// hold 1024 partial pairs
void launch_divergence(const Geom &g, const double *ucont, const double *aj, const double *nvert, double *pv,
                       long long *pi, double *out_v, long long *out_i, cudaStream_t s);
void launch_convection(const Geom &g, const double *ucont, const double *ucat, const double *nvert, int central,
                       double *fp, double *conv, cudaStream_t s);
void launch_metrics_divergence(const Geom &g, const double *csi, const double *eta, const double *zet,
                               const double *aj, double *pv, long long *pi, double *out_v, long long *out_i,
                               cudaStream_t s);
// The momentum right-hand side (kernels_momentum.cu), boxes with no periodic
// face.  fm: the nine face-metric arrays (I, J, K x csi, eta, zet); fp: 9 N
// doubles of scratch; rct: 3 N doubles of scratch.
// gram: the 9 N face metric products of launch_face_gram (formed once per grid)
void launch_face_gram(const Geom &g, const double *const *fm, double *gram, cudaStream_t s);
void launch_viscous(const Geom &g, const double *nvert, const double *ucat, const double *const *fm,
                    const double *iaj, const double *jaj, const double *kaj, const double *gram, double nu,
                    double *fp, double *visc, cudaStream_t s);
void launch_form_function1(const Geom &g, const double *nvert, const double *p, const double *conv,
                           const double *visc, const double *csi, const double *eta, const double *zet,
                           const double *aj, const double *const *fm, const double *iaj, const double *jaj,
                           const double *kaj, const double *gram, double *rct, double *rhs, cudaStream_t s);
void launch_calc_rhs(const Geom &g, const double *nvert, const double *ucont, const double *ucont_o,
                     const double *ucont_rm1, int bdf2, double neg_inv_dt, int mz_end, double *rhs, cudaStream_t s);
// bc: the level's bctype[6]; the host has refused the types it does not cover.
// cent: the cell centres ([N][3]) an annulus face needs; u_bc: the rheology
// plates' velocity
void launch_ghost_node_velocity(const Geom &g, const int *bc, const double *csi, const double *eta,
                                const double *zet, double *ubcs, double *ucat, cudaStream_t s,
                                const double *cent = nullptr, double u_bc = 0.);
// FormBCS with walls on the x and y faces: its three passes of the outlet's
// flux correction (outlet_pass, empty for a walled k = mz - 1 face; it
// launches on s), Contra2Cart, the ghost faces' interior cells and the 12
// edge averages of ucat and p
void launch_form_bcs(const Geom &g, const double *csi, const double *eta, const double *zet, const double *fac,
                     const double *nvert, double *ucont, double *ubcs, double *ucat, double *p,
                     const std::function<void()> &outlet_pass, cudaStream_t s);
// InflowFlux on an inlet k = 0 face with a constant speed uin: ubcs and
// Ucont.z there, and the face's flux terms in the reference's loop order into
// terms ((mx - 2)(my - 2) doubles) for the host to add
void launch_inflow(const Geom &g, const double *nvert, const double *zet, double uin, const double *coor0,
                   int profile, double cmy, double cmz, const double *uin_cell, double *ucont, double *ubcs,
                   double *terms, cudaStream_t s);
// The outlet's flux correction (one FormBCS pass, bctype[5] 4): its flux and
// area terms in the reference's loop order into terms[0 .. n2) and
// terms[n2 .. 2 n2); then, with the ratio the host formed from their sums,
// ubcs on the last face and Ucont.z of the last interior face
void launch_outlet_terms(const Geom &g, const double *nvert, const double *zet, const double *ucat, double *terms,
                         cudaStream_t s);
void launch_outlet_apply(const Geom &g, const double *nvert, const double *zet, const double *ucat, double ratio,
                         double *ucont, double *ubcs, cudaStream_t s);
// ImpRK's stage update u = a rhs + pu, and its two infinity norms (|rhs|,
// |pu - u|; pu null: |rhs| only) as bit patterns into out[0..1] (device)
void launch_imp_waxpy(size_t n, double a, const double *rhs, const double *pu, double *u, cudaStream_t s);
void launch_imp_norms(size_t n, const double *rhs, const double *pu, const double *u, unsigned long long *out,
                      cudaStream_t s);

}  // namespace cvb
