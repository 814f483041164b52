// Tensor-memory-accelerator (TMA) staging helpers for sm_103a: tensor maps over
// a level's arrays, bulk tensor copies into shared memory completed on an
// mbarrier, and bounded waits.
//
// Tensor maps need 16-byte row strides, and a level's rows (mx floats, the
// reference's DMDA box) are not always a multiple of 16 bytes (mx = 258 for
// the channel).  A box with mx even is therefore viewed two rows at a time:
// dimension 0 is a pair of rows (2 mx values, 8 mx bytes), dimension 1 the
// pair index, dimension 2 the plane (mx my values).  Row 2q of a pair starts
// at x = 0, row 2q + 1 at x = mx.  Box starts must be multiples of 4 floats:
// with c a multiple of 4, the even rows' box starts at x = c - 4 and the odd
// rows' at x = mx + c - 4 + odd_shift(mx), which is again a multiple of 4.
// No array is copied or padded for this.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace cvb {

// The two-rows-per-pair view of one [planes][my][mx] FP32 / u32 array.
struct PairView {
  // tensor-map eligibility of a box: rows of even length, an even row count,
  // and plane strides that are multiples of 16 bytes
  __host__ __device__ static bool ok(int mx, int my) { return (mx & 1) == 0 && (my & 1) == 0 && mx >= 4; }
  // shift of the odd rows' box start against the even rows' (in floats): the
  // odd row starts at mx, which is 2 mod 4 when mx is 2 mod 4
  __host__ __device__ static int odd_shift(int mx) { return (mx & 3) == 2 ? 2 : 0; }
};

// Bounded mbarrier wait: gives up after `limit` polls (each try_wait may
// suspend the thread for a while before it returns false).
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int limit) {
  for (int it = 0; it < limit; it++) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// Makes the barrier initialisation visible to the async (TMA) proxy.
__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// One 3-D tensor tile into shared memory (this CTA only, no multicast).
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *map, int c0, int c1, int c2,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
      : "memory");
}

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Host: a pair-view tensor map of a 4-byte array of `planes` planes of
// [my][mx], box {box_x floats, box_pairs pairs, 1 plane}; zero fill outside.
// Returns false if the driver refuses it.
bool tma_pair_map(CUtensorMap *map, const void *base, int mx, int my, int planes, int box_x, int box_pairs);

// Device flag a TMA kernel sets when one of its bounded waits gave up, and its
// host-side check (reads and clears it; synchronises the stream).
int tma_timeout_take(cudaStream_t s);

}  // namespace cvb
