// FP32 factorisation + FP64 refinement instantiations of the perturbation kernel, 1 warp(s) per mode.
#include "sbz_pt_impl.cuh"

namespace sbz {

int pt_launch_f32_w1(const PtArgs& A, int nw, int warps_per_block, int blocks_per_sm, int num_sms, cudaStream_t stream) {
  using namespace ptk;
  switch (nw) {
    case 1:
      switch ((A.model_n + 31) / 32) {
      case 1: return launch_nw<1, 1, float>(A, warps_per_block, blocks_per_sm, num_sms, stream);
      case 2: return launch_nw<1, 2, float>(A, warps_per_block, blocks_per_sm, num_sms, stream);
      case 3: return launch_nw<1, 3, float>(A, warps_per_block, blocks_per_sm, num_sms, stream);
      case 4: return launch_nw<1, 4, float>(A, warps_per_block, blocks_per_sm, num_sms, stream);
      case 5: return launch_nw<1, 5, float>(A, warps_per_block, blocks_per_sm, num_sms, stream);
      case 6: return launch_nw<1, 6, float>(A, warps_per_block, blocks_per_sm, num_sms, stream);
        default: return SBZ_ERR_ARG;
      }
    default: return SBZ_ERR_ARG;
  }
}

}  // namespace sbz
