// The per-block context behind the cvb C ABI, shared by the single-solve host
// code (cvb_api.cpp) and the batch engine (cvb_batch.cpp).
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/cvb.h"
#include "cvb_internal.h"

namespace cvb {

constexpr int kMaxRestart = 64;

struct LevelHost {
  cvb_level_desc d;  // shapes / flags only (pointers are not kept)
};

// The grid's resident metrics, shared by every context built on the same grid
// (cvb_setup_like): problems that differ only in their immersed bodies keep
// one copy.  Freed with its last context.
struct Geometry {
  int device = 0;
  std::vector<void *> allocs;
  size_t bytes = 0;
  std::vector<std::vector<double *>> fm;  // [level][9] raw face metrics (Cmpnts)
  std::vector<double *> iaj, jaj, kaj, aj64;
  double *area3 = nullptr;                // finest: |csi|, |eta|, |zet| per cell ([3][N])
  double *cm[3] = {};                     // finest: centre metrics csi, eta, zet (Cmpnts, [N][3])
  double *inv_aj = nullptr;               // finest: 1 / aj, for the range projection's sum of b / aj
  double *gram = nullptr;                 // finest, on first use: face metric products ([9][N], see k_face_gram)
  double *c2c = nullptr;                  // finest, on first use: Contra2Cart's minors and determinant ([10][N])
  ~Geometry() {
    if (allocs.empty()) return;
    cudaSetDevice(device);
    for (void *p : allocs) cudaFree(p);
  }
};

// A captured V-cycle of one context (see vcycle_graph).
struct VGraph {
  cudaGraphExec_t exec = nullptr;
  int nodes = 0, uses = 0;
  bool failed = false;
  double omega = -1.0;
  int pre = -1, post = -1, smoother = -1;
  const void *b = nullptr;
  void *out = nullptr;
};

}  // namespace cvb

struct cvb_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string err;
  std::vector<void *> allocs;
  std::vector<size_t> alloc_bytes;
  size_t device_bytes = 0;  // sum of this context's device allocations
  size_t device_limit = 0;  // cap on device_bytes + geometry bytes this context allocates (0: none)

  int nlevels = 0;
  std::vector<cvb::LevelDev> L;       // 0 = coarsest
  std::vector<cvb::LevelHost> H;
  // the grid's metrics (shared) and aliases of its arrays
  std::shared_ptr<cvb::Geometry> geo;
  std::vector<std::vector<double *>> fm;  // [level][9] Cmpnts arrays
  std::vector<double *> iaj, jaj, kaj, aj64;
  double *area3 = nullptr;       // finest: |csi|,|eta|,|zet| per cell ([3][N])
  double *cm[3] = {};            // finest: centre metrics csi, eta, zet (Cmpnts)
  double *inv_aj = nullptr;      // finest: 1 / aj (the Geometry's)
  int *cidx = nullptr;           // coarsest level: fluid cells first, then the rest
  double *nvert_tmp = nullptr;
  // coarsest-level solver
  double *Minv = nullptr;
  int ncoarse = 0;
  bool coarse_dense = false;
  int multinullspace = 0;
  std::vector<int> kske;
  // finest-level solver workspace
  double *b = nullptr, *x = nullptr, *w = nullptr, *r = nullptr;
  double *V[cvb::kMaxRestart + 1] = {};
  double *Z64[cvb::kMaxRestart] = {};
  float *Z32[cvb::kMaxRestart] = {};
  float *b32 = nullptr;
  double **dV = nullptr;  // device copies of the pointer tables
  double **dZ64 = nullptr;
  float **dZ32 = nullptr;
  double *partial = nullptr, *sums = nullptr, *hdev = nullptr;
  double *uc_dev = nullptr, *p_dev = nullptr;
  double *ucat_dev = nullptr, *ubcs_dev = nullptr;  // Contra2Cart / GhostNodeVelocity (allocated on first use)
  double *conv_dev = nullptr, *conv_fp = nullptr;    // Convection: result and face fluxes (allocated on first use)
  // momentum right-hand side (Viscous, FormFunction1, CalcRHS; allocated on first use)
  double *visc_dev = nullptr, *rct_dev = nullptr, *rhs_dev = nullptr, *uo_dev = nullptr, *urm_dev = nullptr;
  double *pu_dev = nullptr;                // ImpRK: the last kept iterate (pUcont)
  unsigned long long *imp_norms = nullptr; // ImpRK: |Rhs| and |dU| as bit patterns
  double *inlet_coor = nullptr;  // the k = 0 node plane ([my][mx][3]) for the shaped inlet profiles
  double inlet_cm[3] = {};       // CMx_c, CMy_c, CMz_c
  std::vector<double> inlet_plane_host;  // the same plane on the host (profile 10's speeds)
  double *inlet_uin = nullptr;   // profile 10's speed per inlet face cell ([my - 2][mx - 2]), formed on the host
  bool inlet_uin_ready = false;
  int inlet_uin_key = -1;        // the profile (and table step) inlet_uin holds
  std::vector<double> inlet_table;  // InletRead's uinr [101][1001] (profiles 0 and 5)
  double inlet_flux_in = 4.104388e-04;  // the reference's Flux_in (its initial value), profiles 3 and 6
  int inlet_ti = 0;                     // the time step profile 8 reads
  double *bc_scratch = nullptr;            // InflowFlux / outlet: plane terms (device)
  double *bc_host = nullptr;               // the same terms, pinned host memory, for the host's ordered sums
  double u_bc = 0.;                        // GhostNodeVelocity: the rheology plates' velocity (bcs.c's U_bc)
  double *ibm_cent = nullptr;  // cell centres of the last cvb_ibm_search that gave them
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  bool ready = false;
  // changes with every set-up of the operators (process-wide counter): the
  // batch engine's captured V-cycles are valid for one value
  unsigned long long setup_id = 0;
  // wall-clock ms of the last set-up's phases: metrics upload (0 when the grid
  // was shared), level arrays, operators, autotuner, coarsest solver
  double setup_ms[5] = {};
  std::map<int, cvb::VGraph> vgraphs;  // captured V-cycles by (precision, basis slot)
  // measured sweep times (us): line sweeps fused / split, zebra sweeps two-kernel /
  // one-kernel, and the FP32 zebra sweep with TMA-staged tiles of 4, 8, 16 row
  // pairs (0: not run on this level)
  struct Tune { int level; size_t cells; double us32[2], us64[2], zb32[2], zb64[2], zt32[3], zw32[2]; };
  std::vector<Tune> tune;
};

// Allocates the finest level's FGMRES basis V[0..m], Z[0..m-1] (and the FP32
// V-cycle output in mixed precision) if missing, and refreshes the device tables.
int cvb_ensure_basis(cvb_ctx *ctx, int m, bool mixed);
