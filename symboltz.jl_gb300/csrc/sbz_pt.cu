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
  // four-warp groups: two resident per SM, so the slowest modes share an SM's FP64 pipes with at
  // most one other mode (measured on a 1000-mode spectrum: 0.57 s against 0.70 s at full occupancy)
  if (blocks_per_sm <= 0 && nw == 4) blocks_per_sm = 2;
  if (precision == SBZ_MIXED) {
    // lazy refinement left open: on for four-warp groups (latency-bound: fewer dependent phases
    // per step), off for narrower ones (throughput-bound batches measured 11 % slower with it)
    PtArgs B = A;
    if (B.refine_skip < 0) B.refine_skip = nw == 4 ? 1e-5f : 0.0f;
    return nw == 1 ? pt_launch_f32_w1(B, nw, warps_per_block, blocks_per_sm, num_sms, stream) : pt_launch_f32_w2_w4(B, nw, warps_per_block, blocks_per_sm, num_sms, stream);
  }
  return nw == 1 ? pt_launch_f64_w1(A, nw, warps_per_block, blocks_per_sm, num_sms, stream) : pt_launch_f64_w2_w4(A, nw, warps_per_block, blocks_per_sm, num_sms, stream);
}

}  // namespace sbz
