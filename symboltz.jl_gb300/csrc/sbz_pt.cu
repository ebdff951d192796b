// Precision dispatch of the perturbation kernel (sbz_pt_impl.cuh).
#include "sbz_pt.cuh"

namespace sbz {

int pt_launch_f32(const PtArgs& A, int warps_per_block, int num_sms, cudaStream_t stream);
int pt_launch_f64(const PtArgs& A, int warps_per_block, int num_sms, cudaStream_t stream);

int pt_launch(const PtArgs& A, int precision, int warps_per_block, int num_sms, cudaStream_t stream) {
  if (warps_per_block <= 0) warps_per_block = 4;
  return precision == SBZ_MIXED ? pt_launch_f32(A, warps_per_block, num_sms, stream)
                                : pt_launch_f64(A, warps_per_block, num_sms, stream);
}

}  // namespace sbz
