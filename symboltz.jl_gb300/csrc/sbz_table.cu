// Device build of the background coefficient tables: one thread per (cosmology, node), the same
// table_node arithmetic as the host build, written straight into the layout the perturbation
// kernels read (τ_g, 1/(τ_{g+1} - τ_g), the kTabValues values, then the power-form interpolation
// coefficients of the node's interval; kNodeStride doubles per node).
// Only the background knots and node times cross the bus (≈ 100 KB per cosmology instead of the
// 1 MB table), and the ~14 µs of Taylor-mode work per node leaves the host.
#include <cuda_runtime.h>
#include "sbz_layout.hpp"
#include "sbz_table.cuh"
#include "../../include/symboltz_gb300.h"

namespace sbz {

static_assert(kNodePow >= 2 + kTabValues && kNodePow + 2 * kTabValues <= kNodeStride, "table node layout");

namespace {

__global__ void __launch_bounds__(128) table_kernel(int ntab, int ncos, const Cosmo* __restrict__ P, const BgKnot* __restrict__ knots,
                                                    const int* __restrict__ koff, const int* __restrict__ nknot,
                                                    const double* __restrict__ kappa0, const double* __restrict__ tabtau,
                                                    const int* __restrict__ ok, double* __restrict__ tab, long long stride) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= (long long)ntab * ncos) return;
  const int c = (int)(i / ntab), g = (int)(i - (long long)c * ntab);
  double* nd = tab + (long long)c * stride + (long long)g * kNodeStride;
  if (!ok[c]) {  // failed background: a flat dummy table (the kernels never read it)
    for (int q = 0; q < kNodeStride; ++q) nd[q] = 0.0;
    return;
  }
  const double* tt = tabtau + (long long)c * ntab;
  const double tau = tt[g];
  nd[0] = tau;
  nd[1] = (g + 1 < ntab) ? 1.0 / (tt[g + 1] - tau) : 0.0;
  table_node(P[c], knots + koff[c], nknot[c], kappa0[c], tau, nd + 2);
}

// Power form of each quantity's cubic Hermite interpolant on [τ_g, τ_{g+1}] from the two nodes'
// (value, d/dτ) pairs: p(s) = a0 + a1 s + a2 s² + a3 s³, a0 = v0, a1 = h d0,
// a2 = 3 (v1 - v0) - h (2 d0 + d1), a3 = h (d0 + d1) - 2 (v1 - v0), h = τ_{g+1} - τ_g (the Hermite
// basis expanded in powers of s), so the perturbation kernels evaluate a value with three FMAs.
__global__ void __launch_bounds__(128) table_pow_kernel(int ntab, int ncos, const int* __restrict__ ok, double* __restrict__ tab,
                                                        long long stride) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= (long long)ntab * ncos) return;
  const int c = (int)(i / ntab), g = (int)(i - (long long)c * ntab);
  double* nd = tab + (long long)c * stride + (long long)g * kNodeStride;
  double* P = nd + kNodePow;
  if (!ok[c] || g + 1 >= ntab) {
    for (int q = 0; q < 4 * kTabValues / 2; ++q) P[q] = 0.0;
    return;
  }
  const double* nx = nd + kNodeStride;
  const double h = nx[0] - nd[0];
  for (int j = 0; j < kTabValues / 2; ++j) {
    const double v0 = nd[2 + 2 * j], d0 = nd[3 + 2 * j], v1 = nx[2 + 2 * j], d1 = nx[3 + 2 * j];
    const double dv = v1 - v0;
    P[4 * j] = v0;
    P[4 * j + 1] = h * d0;
    P[4 * j + 2] = 3 * dv - h * (2 * d0 + d1);
    P[4 * j + 3] = h * (d0 + d1) - 2 * dv;
  }
}

}  // namespace

int table_build_launch(int ntab, int ncos, const Cosmo* d_cosmo, const BgKnot* d_knots, const int* d_koff, const int* d_nknot,
                       const double* d_kappa0, const double* d_tabtau, const int* d_ok, double* d_tab, long long stride,
                       cudaStream_t stream) {
  const long long n = (long long)ntab * ncos;
  if (n <= 0) return SBZ_OK;
  const int threads = 128;
  const long long blocks = (n + threads - 1) / threads;
  table_kernel<<<(unsigned)blocks, threads, 0, stream>>>(ntab, ncos, d_cosmo, d_knots, d_koff, d_nknot, d_kappa0, d_tabtau, d_ok, d_tab,
                                                          stride);
  table_pow_kernel<<<(unsigned)blocks, threads, 0, stream>>>(ntab, ncos, d_ok, d_tab, stride);
  return cudaGetLastError() == cudaSuccess ? SBZ_OK : SBZ_ERR_CUDA;
}

}  // namespace sbz
