// all-FP64 instantiations of the perturbation kernel, 1 warp(s) per mode.
#include "sbz_pt_impl.cuh"

namespace sbz {

int pt_launch_f64_w1(const PtArgs& A, int nw, int warps_per_block, int blocks_per_sm, int num_sms, cudaStream_t stream) {
  using namespace ptk;
  switch (nw) {
    case 1:
      switch ((A.model_n + 31) / 32) {
      case 1: return launch_nw<1, 1, double>(A, warps_per_block, blocks_per_sm, num_sms, stream);
      case 2: return launch_nw<1, 2, double>(A, warps_per_block, blocks_per_sm, num_sms, stream);
      case 3: return launch_nw<1, 3, double>(A, warps_per_block, blocks_per_sm, num_sms, stream);
      case 4: return launch_nw<1, 4, double>(A, warps_per_block, blocks_per_sm, num_sms, stream);
      case 5: return launch_nw<1, 5, double>(A, warps_per_block, blocks_per_sm, num_sms, stream);
      case 6: return launch_nw<1, 6, double>(A, warps_per_block, blocks_per_sm, num_sms, stream);
        default: return SBZ_ERR_ARG;
      }
    default: return SBZ_ERR_ARG;
  }
}

int rhs_launch(const PtArgs& A, const double* y, const double* tau, double* f, double* ft, cudaStream_t st) {
  using namespace ptk;
  switch ((A.model_n + 31) / 32) {
    case 1: return rhs_launch_ns<1>(A, y, tau, f, ft, st);
    case 2: return rhs_launch_ns<2>(A, y, tau, f, ft, st);
    case 3: return rhs_launch_ns<3>(A, y, tau, f, ft, st);
    case 4: return rhs_launch_ns<4>(A, y, tau, f, ft, st);
    case 5: return rhs_launch_ns<5>(A, y, tau, f, ft, st);
    case 6: return rhs_launch_ns<6>(A, y, tau, f, ft, st);
    default: return SBZ_ERR_ARG;
  }
}

}  // namespace sbz
