// One zebra half-sweep of the FP32 V-cycle with its inputs staged by the
// tensor memory accelerator: the y-line smoother's hot kernel on levels
// without cross-derivative terms (the channel's 7-point rows).
//
// A block takes kTmaLines lines of one colour in one plane k (columns
// [16 bx, 16 bx + 16)), as the one-kernel form in stencil_body.cuh does, and
// walks down the rows in chunks of RP row pairs.  For every chunk one thread
// issues 20 bulk tensor copies -- x on planes k-1, k, k+1, g11, g22, g33 and aj,
// code, b on plane k, and g33 on plane k-1, each as two boxes (even and odd
// rows, PairView) of 24 columns with a one-pair halo above and below -- into
// one of two shared-memory stages, completed on that stage's mbarrier.  While
// the next chunk is in flight the block forms the colour's 7-point residuals
// of the current one from shared memory into the line tile.  The line solves
// and the in-place update then follow as in the one-kernel form (Thomas
// factors in registers, R <= 4 rows per lane).
//
// Every wait is bounded: a wait that gives up sets g_tma_timeout, waits (with
// a bound) for the stage's other copies, and the block returns without
// writing; the host turns the flag into CVB_TIMEOUT.
#include <mutex>
#include <unordered_map>

#include "stencil_body.cuh"
#include "tma.cuh"

namespace cvb {

__device__ int g_tma_timeout;

namespace {

constexpr int kTmaLines = kSolveTW32;  // 8 lines per tile: 16 columns
constexpr int kBoxX = 24;              // columns staged per row: [c0 - 4, c0 + 20)
constexpr int kArrays = 10;            // x(k-1), x(k), x(k+1), g11, g22, g33, g33(k-1), aj, code, b
constexpr int kWaitPolls = 1 << 22;    // bound of one mbarrier wait (about a second)

enum { AX_B = 0, AX_P = 1, AX_T = 2, AG11 = 3, AG22 = 4, AG33 = 5, AG33B = 6, AAJ = 7, ACODE = 8, ARHS = 9 };

// floats of one [array][row parity] slab of a stage: RP + 2 pairs of kBoxX
// columns, rounded up to 128 bytes (the copies' destination alignment)
template <int RP>
__host__ __device__ constexpr int slab_floats() { return ((kBoxX * (RP + 2)) + 31) & ~31; }
template <int RP>
__host__ __device__ constexpr int stage_floats() { return kArrays * 2 * slab_floats<RP>(); }
template <int RP>
__host__ __device__ constexpr uint32_t stage_bytes() { return kArrays * 2 * kBoxX * (RP + 2) * 4; }  // transferred per chunk

struct TmaMaps {
  CUtensorMap x, b, g, aj, code;
};

}  // namespace

// Shared memory of one block: two stages, then the line tile (residual and x
// of the colour's lines, LineLayout), then two mbarriers.
template <int RP>
inline size_t zebra_tma_smem(const Geom &g) {
  const LineLayout Lo = LineLayout::of(g.my);
  return sizeof(float) * (2 * (size_t)stage_floats<RP>() + 2 * (size_t)Lo.ls * kTmaLines) + 16 + 128;
}

template <int RP, int RR>
__global__ void __launch_bounds__(kSolveThreads) k_zebra_tma(const __grid_constant__ LevelDev L,
                                                             const __grid_constant__ TmaMaps M, float *x, float omega,
                                                             int color) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  dep_sync();
  if (gated(L.gate)) return;
  const Geom &g = L.g;
  const int k = blockIdx.y, bx = blockIdx.x;
  if (k < 1 || k > g.mz - 2) return;
  const int mx = g.mx, my = g.my;
  const int c0 = 2 * kTmaLines * bx, par = (color + k) & 1;
  const int oshift = PairView::odd_shift(mx);
  // 128-byte aligned stages
  float *base = reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  float *stage[2] = {base, base + stage_floats<RP>()};
  const LineLayout Lo = LineLayout::fixed<RR>(my);
  float *sr = base + 2 * stage_floats<RP>(), *sx = sr + Lo.ls * kTmaLines;
  uint64_t *bars = reinterpret_cast<uint64_t *>(sx + Lo.ls * kTmaLines);
  const uint32_t bar0 = smem_addr(&bars[0]), bar1 = smem_addr(&bars[1]);
  const int npairs = my >> 1, nchunks = (npairs + RP - 1) / RP;
  const int kb = (g.pz && k == 1) ? g.mz - 2 : k - 1, kt = (g.pz && k == g.mz - 2) ? 1 : k + 1;
  if (threadIdx.x == 0) {
    mbar_init(bar0, 1);
    mbar_init(bar1, 1);
    fence_barrier_init();
  }
  __syncthreads();
  // one chunk's 20 copies into stage st (thread 0)
  auto issue = [&](int s, int st) {
    const uint32_t bar = st ? bar1 : bar0;
    mbar_expect_tx(bar, stage_bytes<RP>());
    const int q = s * RP - 1;
    float *dst = stage[st];
    const int xe = c0 - 4, xo = mx + c0 - 4 + oshift;
    const int nz = g.mz;
    const CUtensorMap *maps[kArrays] = {&M.x, &M.x, &M.x, &M.g, &M.g, &M.g, &M.g, &M.aj, &M.code, &M.b};
    const int planes[kArrays] = {kb, k, kt, k, 4 * nz + k, 8 * nz + k, 8 * nz + k - 1, k, k, k};
#pragma unroll
    for (int a = 0; a < kArrays; a++) {
      tma_load_3d(smem_addr(dst + (2 * a) * slab_floats<RP>()), maps[a], xe, q, planes[a], bar);
      tma_load_3d(smem_addr(dst + (2 * a + 1) * slab_floats<RP>()), maps[a], xo, q, planes[a], bar);
    }
  };
  if (threadIdx.x == 0) {
    issue(0, 0);
    if (nchunks > 1) issue(1, 1);
  }
  int failed = -1;  // the chunk whose wait gave up (the same in every thread)
  const int px = g.px;
  for (int s = 0; s < nchunks; s++) {
    const int st = s & 1;
    const bool landed = mbar_wait(st ? bar1 : bar0, (s >> 1) & 1, kWaitPolls);
    if (!__syncthreads_and(landed)) {
      failed = s;
      break;
    }
    const float *S = stage[st];
    const int jlo = 2 * s * RP, jhi = min(2 * (s + 1) * RP, my);  // rows of this chunk
    // value of array a at (row j, column i) of this chunk
    auto at = [&](int a, int j, int i) -> float {
      const int pj = j & 1, qq = (j >> 1) - (s * RP - 1);
      const int col = i - (c0 - 4) - (pj ? oshift : 0);
      return S[(2 * a + pj) * slab_floats<RP>() + qq * kBoxX + col];
    };
    for (int e = threadIdx.x; e < kTmaLines * (jhi - jlo); e += kSolveThreads) {
      const int t = e % kTmaLines, j = jlo + e / kTmaLines;
      const int i = c0 + 2 * t + par;
      if (j < 1 || j > my - 2 || i < 1 || i > mx - 2) continue;
      const uint32_t c = __float_as_uint(at(ACODE, j, i));
      const float P = at(AX_P, j, i);
      // x across a periodic seam in i comes from memory (the other colour, which
      // no block writes in this half-sweep)
      const int p = (k * my + j) * mx + i;
      const float E = (px && i == mx - 2) ? x[p - (mx - 3)] : at(AX_P, j, i + 1);
      const float W = (px && i == 1) ? x[p + (mx - 3)] : at(AX_P, j, i - 1);
      const float N = at(AX_P, j + 1, i), Sv = at(AX_P, j - 1, i);
      const float T = at(AX_T, j, i), B = at(AX_B, j, i);
      const float g11 = at(AG11, j, i), w11 = at(AG11, j, i - 1);
      const float g22 = at(AG22, j, i), s22 = at(AG22, j - 1, i);
      const float g33 = at(AG33, j, i), b33 = at(AG33B, j, i);
      const float ajp = at(AAJ, j, i), bp = at(ARHS, j, i);
      // row32<float, false>: the same flux form in the same order
      const float fe = g11 * (E - P), fw = w11 * (P - W), fn = g22 * (N - P);
      const float fs = s22 * (P - Sv), ft = g33 * (T - P), fb = b33 * (P - B);
      const float acc = act(c, CODE_ACT_E) * fe - act(c, CODE_ACT_W) * fw + act(c, CODE_ACT_N) * fn -
                        act(c, CODE_ACT_S) * fs + act(c, CODE_ACT_T) * ft - act(c, CODE_ACT_B) * fb;
      const float ax = (c & CODE_IDENTITY) ? P : -ajp * acc;
      const int o = t * Lo.ls + Lo.pos(j - 1);
      sr[o] = bp - ax;
      sx[o] = P;
    }
    __syncthreads();  // the stage has been read: it may be refilled
    if (threadIdx.x == 0 && s + 2 < nchunks) issue(s + 2, st);
  }
  if (failed >= 0) {
    if (threadIdx.x == 0) atomicExch(&g_tma_timeout, 1);
    // let the copies still in flight (chunks failed and failed + 1) land before
    // the block's shared memory is released, again with a bound
    for (int s = failed; s < min(failed + 2, nchunks); s++) mbar_wait((s & 1) ? bar1 : bar0, (s >> 1) & 1, kWaitPolls);
    return;
  }
  TileLaneFactors<float, kTmaLines, RR> lf;
  lane_factors_load<float, kTmaLines, RR>(L, bx, k, color, lf);
  constexpr int NW = kSolveThreads / 32, NL = kTmaLines / NW;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  warp_lines_solve<float, NL, RR>(sr + warp * Lo.ls, lf, NW * Lo.ls, Lo, lane);
  __syncthreads();
  const int tx = threadIdx.x % kTmaLines, ty = threadIdx.x / kTmaLines;
  constexpr int ny = kSolveThreads / kTmaLines;
  const int i = c0 + 2 * tx + par;
  if (i < 1 || i > mx - 2) return;
  const int col = (k * my) * mx + i;
  for (int j = 1 + ty; j <= my - 2; j += ny) {
    const int o = tx * Lo.ls + Lo.pos(j - 1);
    x[col + j * mx] = sx[o] + omega * sr[o];
  }
}

// ------------------------------------------------------------------ host side
namespace {

using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encoder() {
  static EncodeTiled fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return static_cast<EncodeTiled>(nullptr);
    return reinterpret_cast<EncodeTiled>(p);
  }();
  return fn;
}

struct MapKey {
  const void *p;
  int mx, my, planes, box_pairs;
  bool operator==(const MapKey &o) const {
    return p == o.p && mx == o.mx && my == o.my && planes == o.planes && box_pairs == o.box_pairs;
  }
};
struct MapKeyHash {
  size_t operator()(const MapKey &k) const {
    return std::hash<const void *>()(k.p) ^ ((size_t)k.mx * 1000003u + (size_t)k.my * 10007u + k.planes * 31u +
                                             k.box_pairs);
  }
};
std::mutex g_map_mu;
std::unordered_map<MapKey, CUtensorMap, MapKeyHash> g_maps;

bool cached_map(CUtensorMap *out, const void *p, int mx, int my, int planes, int box_pairs) {
  const MapKey key{p, mx, my, planes, box_pairs};
  std::lock_guard<std::mutex> lock(g_map_mu);
  auto it = g_maps.find(key);
  if (it != g_maps.end()) {
    *out = it->second;
    return true;
  }
  if (!tma_pair_map(out, p, mx, my, planes, kBoxX, box_pairs)) return false;
  if (g_maps.size() > 4096) g_maps.clear();
  g_maps.emplace(key, *out);
  return true;
}

}  // namespace

bool tma_pair_map(CUtensorMap *map, const void *base, int mx, int my, int planes, int box_x, int box_pairs) {
  EncodeTiled enc = encoder();
  if (!enc || !PairView::ok(mx, my) || (reinterpret_cast<uintptr_t>(base) & 15)) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)2 * mx, (cuuint64_t)(my / 2), (cuuint64_t)planes};
  const cuuint64_t strides[2] = {(cuuint64_t)2 * mx * 4, (cuuint64_t)mx * my * 4};
  const cuuint32_t box[3] = {(cuuint32_t)box_x, (cuuint32_t)box_pairs, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void *>(base), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int tma_timeout_take(cudaStream_t s) {
  int h = 0;
  if (cudaMemcpyFromSymbolAsync(&h, g_tma_timeout, sizeof(int), 0, cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return -1;
  if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
  if (h) {
    const int zero = 0;
    cudaMemcpyToSymbolAsync(g_tma_timeout, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, s);
    cudaStreamSynchronize(s);
  }
  return h;
}

// Whether the TMA half-sweep can run on a level: FP32 7-point rows in place
// (zebra_fusable), a pair view of the box, no periodic wrap in y, R <= 4 rows
// per lane, and room for the pair count in one box dimension.
bool zebra_tma_ok(const LevelDev &L) {
  const Geom &g = L.g;
  return zebra_fusable<float>(L) && PairView::ok(g.mx, g.my) && !g.py && LineLayout::of(g.my).R <= 4 &&
         g.my / 2 <= 256 && encoder() != nullptr;
}

template <int RP, int RR>
static bool zebra_tma_rr(const LevelDev &L, const float *b, float *x, float omega, int color, cudaStream_t s) {
  const Geom &g = L.g;
  TmaMaps M;
  if (!cached_map(&M.x, x, g.mx, g.my, g.mz, RP + 2) || !cached_map(&M.b, b, g.mx, g.my, g.mz, RP + 2) ||
      !cached_map(&M.g, L.gf32, g.mx, g.my, 9 * g.mz, RP + 2) ||
      !cached_map(&M.aj, L.ajf32, g.mx, g.my, g.mz, RP + 2) ||
      !cached_map(&M.code, L.code, g.mx, g.my, g.mz, RP + 2))
    return false;
  static bool attr = false;
  const size_t smem = zebra_tma_smem<RP>(g);
  if (!attr) {
    cudaFuncSetAttribute(k_zebra_tma<RP, RR>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attr = true;
  }
  dim3 grd(solve_tiles_x<kTmaLines>(g, color), g.mz);
  launch_dep(k_zebra_tma<RP, RR>, grd, kSolveThreads, smem, s, L, M, x, omega, color);
  return true;
}

template <int RP>
static bool zebra_tma_r(const LevelDev &L, const float *b, float *x, float omega, int color, cudaStream_t s) {
  switch (LineLayout::of(L.g.my).R) {
    case 1: return zebra_tma_rr<RP, 1>(L, b, x, omega, color, s);
    case 2: return zebra_tma_rr<RP, 2>(L, b, x, omega, color, s);
    case 4: return zebra_tma_rr<RP, 4>(L, b, x, omega, color, s);
    default: return false;
  }
}

// The TMA half-sweep with chunks of rp row pairs (4, 8 or 16: the tile shape
// the set-up autotuner picks); false when it cannot run here (the caller then
// takes another form).
bool launch_zebra_tma(const LevelDev &L, const float *b, float *x, float omega, int color, int rp, cudaStream_t s) {
  if (!zebra_tma_ok(L)) return false;
  switch (rp) {
    case 4: return zebra_tma_r<4>(L, b, x, omega, color, s);
    case 8: return zebra_tma_r<8>(L, b, x, omega, color, s);
    case 16: return zebra_tma_r<16>(L, b, x, omega, color, s);
    default: return false;
  }
}

}  // namespace cvb
