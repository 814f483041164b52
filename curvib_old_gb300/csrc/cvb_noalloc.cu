// PoissonRHS on caller-owned device arrays with no device allocation at all.
//
// For callers that cannot call cudaMalloc: hosts whose device memory is handed
// out by their own allocator (a PETSc or framework memory pool) and must not be
// fragmented or exceeded behind the pool's back, and time-stepping loops that
// forbid allocation after start-up so that a long run cannot fail half-way on
// memory.  Inputs and outputs are passed in; the only scratch -- one slot per
// reduction block for the compatibility sum -- is the file-scope array below,
// which every GPU that loads this library holds until the process exits.
#include <cuda.h>

#include <mutex>

#include "../../include/cvb.h"
#include "cvb_internal.h"

namespace {

// Two rows (the reduction writes a pair of sums per block) of one slot per block.
static __device__ __align__(256) double g_rhs_scratch[2 * CVB_NOALLOC_MAX_BLOCKS];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
struct ScratchAddr {
  CUcontext ctx = nullptr;  // the context the address belongs to
  double *ptr = nullptr;
};
ScratchAddr g_scratch[kMaxDevices];

// Device address of g_rhs_scratch in the current context.  In host code the
// symbol is only a host-side stand-in; a kernel must be given this address.
// The lookup runs once per device (the first call there, with that device
// current) and again only if the device's context was replaced since
// (cudaDeviceReset and a new primary context can load the module elsewhere).
int scratch_for_current_device(double **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return CVB_CUDA_ERROR;
  // binds the device's primary context to this thread (CUDA 12+ initialises it here)
  if (cudaSetDevice(dev) != cudaSuccess) return CVB_CUDA_ERROR;
  std::lock_guard<std::mutex> lock(g_mu);
  // cuCtxGetCurrent through the runtime's driver entry point: the library
  // does not link the driver library itself
  static CUresult (*get_current)(CUcontext *) = nullptr;
  if (!get_current) {
    cudaDriverEntryPointQueryResult q;
    void *fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
      return CVB_CUDA_ERROR;
    get_current = reinterpret_cast<CUresult (*)(CUcontext *)>(fn);
  }
  CUcontext cur = nullptr;
  if (get_current(&cur) != CUDA_SUCCESS || !cur) return CVB_CUDA_ERROR;
  ScratchAddr &a = g_scratch[dev];
  if (!a.ptr || a.ctx != cur) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_rhs_scratch);
    if (e != cudaSuccess || !p) return CVB_CUDA_ERROR;
    a.ptr = static_cast<double *>(p);
    a.ctx = cur;
  }
  *out = a.ptr;
  return CVB_OK;
}

}  // namespace

extern "C" int cvb_poisson_rhs_noalloc(const double *d_ucont, const double *d_aj, const double *d_nvert, int mx,
                                       int my, int mz, double dt, double st, double *d_b, double *d_compat_sum,
                                       void *stream) {
  if (!d_ucont || !d_aj || !d_nvert || !d_b || !d_compat_sum) return CVB_BAD_INPUT;
  if (mx < 3 || my < 3 || mz < 3 || !(dt != 0.0) || !(st != 0.0)) return CVB_BAD_INPUT;
  if ((long long)mx * my * mz > (long long)CVB_NOALLOC_MAX_CELLS) return CVB_BAD_INPUT;
  const int nb = cvb::reduce_blocks();
  if (nb > CVB_NOALLOC_MAX_BLOCKS) return CVB_BAD_INPUT;
  double *scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc != CVB_OK) return rc;
  cvb::Geom g;
  g.mx = mx; g.my = my; g.mz = mz;
  g.px = g.py = g.pz = 0;  // PoissonRHS reads no periodic image
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // same kernels, block count and summation tree as cvb_poisson_rhs
  cvb::launch_poisson_rhs(g, d_ucont, d_aj, d_nvert, dt, st, d_b, scratch, s);
  cvb::launch_finish_sums(scratch, 1, nb, d_compat_sum, s);
  return cudaGetLastError() == cudaSuccess ? CVB_OK : CVB_CUDA_ERROR;
}
