// FP32 factorisation + FP64 refinement instantiations of the perturbation kernel, 2, 4 and 8 warps per mode.
#include "sbz_pt_impl.cuh"

namespace sbz {

int pt_launch_f32_w2_w4(const PtArgs& A, int nw, int warps_per_block, int blocks_per_sm, int num_sms, cudaStream_t stream) {
  using namespace ptk;
  switch (nw) {
    case 2:
      switch ((A.model_n + 63) / 64) {
      case 1: return launch_nw<2, 1, float>(A, warps_per_block, blocks_per_sm, num_sms, stream);
      case 2: return launch_nw<2, 2, float>(A, warps_per_block, blocks_per_sm, num_sms, stream);
      case 3: return launch_nw<2, 3, float>(A, warps_per_block, blocks_per_sm, num_sms, stream);
        default: return SBZ_ERR_ARG;
      }
    case 4:
      switch ((A.model_n + 127) / 128) {
      case 1: return launch_nw<4, 1, float>(A, warps_per_block, blocks_per_sm, num_sms, stream);
      case 2: return launch_nw<4, 2, float>(A, warps_per_block, blocks_per_sm, num_sms, stream);
        default: return SBZ_ERR_ARG;
      }
    case 8:
      switch ((A.model_n + 255) / 256) {
      case 1: return launch_nw<8, 1, float>(A, warps_per_block, blocks_per_sm, num_sms, stream);
        default: return SBZ_ERR_ARG;
      }
    default: return SBZ_ERR_ARG;
  }
}

}  // namespace sbz
