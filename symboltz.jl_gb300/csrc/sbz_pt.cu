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
  if (nw != 1 && nw != 2 && nw != 4) return SBZ_ERR_ARG;
  // four-warp groups: a spectrum of up to 8 modes per SM is set by its slowest modes, which then
  // get an SM's FP64 pipes to themselves (one group per SM; measured on the 1000-mode spectrum at
  // rtol 1e-6, atol 3e-8: 2.99 s against 3.70 s with two groups per SM); larger launches keep two
  // groups per SM, so a slow mode shares its SM with at most one other
  if (blocks_per_sm <= 0 && nw == 4) blocks_per_sm = A.nitems <= 8 * num_sms ? 1 : 2;
  if (precision == SBZ_MIXED) {
    // refinement left open: stage 1 only.  Its FP64 correction covers the step's conditioning
    // (stage 1 has the largest right-hand side); the later stages' FP32 solves then differ from the
    // refined ones far below the tolerance (measured C_l 3.9e-6 from the all-FP64 solver on the
    // 1000-mode spectrum at rtol 1e-6, atol 3e-8, at 0.69x the time of refining every stage)
    PtArgs B = A;
    if (B.refine_skip < 0) B.refine_skip = 3.0e38f;
    return nw == 1 ? pt_launch_f32_w1(B, nw, warps_per_block, blocks_per_sm, num_sms, stream) : pt_launch_f32_w2_w4(B, nw, warps_per_block, blocks_per_sm, num_sms, stream);
  }
  return nw == 1 ? pt_launch_f64_w1(A, nw, warps_per_block, blocks_per_sm, num_sms, stream) : pt_launch_f64_w2_w4(A, nw, warps_per_block, blocks_per_sm, num_sms, stream);
}

}  // namespace sbz
