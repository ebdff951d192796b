// FP32 factorisation + FP64 refinement instantiations of the perturbation kernel.
#include "sbz_pt_impl.cuh"

namespace sbz {

int pt_launch_f32(const PtArgs& A, int warps_per_block, int num_sms, cudaStream_t stream) {
  using namespace ptk;
  switch ((A.model_n + 31) / 32) {
    case 1: return launch_ns<1, float>(A, warps_per_block, num_sms, stream);
    case 2: return launch_ns<2, float>(A, warps_per_block, num_sms, stream);
    case 3: return launch_ns<3, float>(A, warps_per_block, num_sms, stream);
    case 4: return launch_ns<4, float>(A, warps_per_block, num_sms, stream);
    case 5: return launch_ns<5, float>(A, warps_per_block, num_sms, stream);
    case 6: return launch_ns<6, float>(A, warps_per_block, num_sms, stream);
    default: return SBZ_ERR_ARG;
  }
}

}  // namespace sbz
