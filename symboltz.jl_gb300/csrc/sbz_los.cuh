// Launch interface of the line-of-sight kernels (sbz_los.cu).
#pragma once
#include <cuda_runtime.h>

namespace sbz {

struct BesselDev {
  double* y;    // [ix * nl + il]
  double* dy;   // same layout, or nullptr for linear interpolation
  float2* yf2;  // FP32 copy (j_l, j_l') interleaved, same layout (mixed-precision line of sight)
  int nl, nx;   // nx includes the duplicated last point
  double xmax, step, invdx, dx;
  int hermite;
};

int bessel_build(BesselDev& J, const int* d_ls, int Lmax, cudaStream_t st);
int bessel_f32_build(const BesselDev& J, cudaStream_t st);
// FP32 line of sight (interpolation and chunk sums in FP32, chunk totals in FP64); il_limber ≤ 1024
int los_f32_launch(const BesselDev& J, const int* d_ls, int nsrc, const double* d_S, const double* d_taus, const double* d_chi,
                   const double* d_w, int ntau, int nk, const double* d_ks, int il_limber, double* d_out, cudaStream_t st);
// C_l[q*nl + il] = Σ_k g_k Θ_a(k,l) Θ_b(k,l) with g_k the spline-integral weights times 2/π k² P0
int cl_dot_launch(int nk, const double* d_g, int nl, int ns, const double* d_Th, int npair, const int* d_pa, const int* d_pb,
                  double* d_Cl, cudaStream_t st);
int bessel_eval(const BesselDev& J, int il, int n, const double* d_x, double* d_out, cudaStream_t st);
int los_launch(const BesselDev& J, const int* d_ls, int nsrc, const double* d_S, const double* d_taus,
               const double* d_chi, const double* d_w, int ntau, int nk, const double* d_ks, int il_limber,
               double* d_out, cudaStream_t st);
int cl_launch(int nk, const double* d_ks, const double* d_P0, int nl, const double* d_ThA, const double* d_ThB,
              const double* d_cprime, const double* d_invden, double* d_zbuf, double* d_Cl, cudaStream_t st);

int kinterp_spline_launch(int nc, int ntau, int ns, int nf, const int* d_src, const double* d_Sc, const double* d_y,
                          const double* d_yf, const int* d_iv, const double* d_cprime, const double* d_invden, double* d_z,
                          double* d_Sf, cudaStream_t st);
int kinterp_bary_launch(int nc, int ntau, int ns, int nf, const int* d_src, const double* d_Sc, const double* d_M, double* d_Sf,
                        cudaStream_t st);
int theta_scale_launch(int nk, int nl, int ns, const double* d_ks, const int* d_ls, int sT, int sE, double* d_Th, cudaStream_t st);

}  // namespace sbz
