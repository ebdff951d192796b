// Precision and group-size dispatch of the perturbation kernel (sbz_pt_impl.cuh).
#include "sbz_pt.cuh"

namespace sbz {

int pt_launch_f32_w1(const PtArgs& A, int nw, int warps_per_block, int blocks_per_sm, int num_sms, cudaStream_t stream);
int pt_launch_f32_w2_w4(const PtArgs& A, int nw, int warps_per_block, int blocks_per_sm, int num_sms, cudaStream_t stream);
int pt_launch_f64_w1(const PtArgs& A, int nw, int warps_per_block, int blocks_per_sm, int num_sms, cudaStream_t stream);
int pt_launch_f64_w2_w4(const PtArgs& A, int nw, int warps_per_block, int blocks_per_sm, int num_sms, cudaStream_t stream);

// Warps per mode when the caller leaves it open: a spectrum's run time is set by its slowest
// (highest-k) modes, so while the modes fit on the GPU a few at a time, each gets the four
// sub-partitions of an SM; large batches keep one warp per mode (no barrier overhead).
static int auto_warps_per_mode(int nitems, int num_sms) { return nitems <= 32 * num_sms ? 4 : 1; }

int pt_launch(const PtArgs& A, int precision, int warps_per_block, int warps_per_mode, int blocks_per_sm, int num_sms,
              cudaStream_t stream) {
  if (warps_per_block <= 0) warps_per_block = 4;
  const int nw = warps_per_mode > 0 ? warps_per_mode : auto_warps_per_mode(A.nitems, num_sms);
  if (nw != 1 && nw != 2 && nw != 4 && nw != 8) return SBZ_ERR_ARG;
  // four-warp groups: a spectrum of up to 8 modes per SM is set by its slowest modes, which then
  // get an SM's FP64 pipes to themselves (one group per SM; measured on the 1000-mode spectrum at
  // rtol 1e-6, atol 3e-8: 2.99 s against 3.70 s with two groups per SM); larger launches keep two
  // groups per SM, so a slow mode shares its SM with at most one other
  if (blocks_per_sm <= 0 && nw == 4) blocks_per_sm = A.nitems <= 8 * num_sms ? 1 : 2;
  if (nw == 8) blocks_per_sm = 1;  // eight-warp groups: one mode per SM
  if (precision == SBZ_MIXED) {
    // lazy refinement left open: the later stages skip their FP64 refinement when stage 1's first
    // correction is below 1e-5 error weights (Rodas5P's stage right-hand sides carry coefficients up
    // to 165, so an unrefined FP32 stage solve stays below the refinement's own 1e-3 stopping level
    // only when stage 1's was well below 1e-5); on for four-warp groups (latency-bound), off for
    // narrower ones (throughput-bound batches).  Skipping the later stages' refinement outright was
    // measured to leave pointwise sources 0.48 (rtol 1e-5) and 1.1e-2 (rtol 1e-7) of their maximum
    // away from the oracle on the reference's ΛCDM(lmax = 5) model.
    PtArgs B = A;
    if (B.refine_skip < 0) B.refine_skip = nw >= 4 ? 1e-5f : 0.0f;
    return nw == 1 ? pt_launch_f32_w1(B, nw, warps_per_block, blocks_per_sm, num_sms, stream)
                   : pt_launch_f32_w2_w4(B, nw, warps_per_block, blocks_per_sm, num_sms, stream);
  }
  return nw == 1 ? pt_launch_f64_w1(A, nw, warps_per_block, blocks_per_sm, num_sms, stream) : pt_launch_f64_w2_w4(A, nw, warps_per_block, blocks_per_sm, num_sms, stream);
}

}  // namespace sbz
