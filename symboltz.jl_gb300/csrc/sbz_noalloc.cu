// C_l integration that allocates no device memory: sbz_cl_integrate_noalloc.
//
// Who needs it: callers whose device memory is owned by their own pool (a Julia program on
// CUDA.jl's allocator, a PyTorch process on its caching allocator, a service with a fixed memory
// budget) and that therefore must not have a library call cudaMalloc/cudaFree behind their back:
// those calls take memory outside the pool's accounting and synchronise the whole device.  They
// pass device buffers for every input and the output; the spline scratch (Thomas factors and the
// per-multipole second-derivative sweep) lives in the fixed array below instead of in allocations.
//
// Rules of use:
//  * Scratch is SBZ_NOALLOC_SCRATCH_DOUBLES doubles (16 MiB); sizes that do not fit are rejected
//    with SBZ_ERR_ARG before any GPU work.
//  * Every call shares the one array per device and it keeps the previous call's contents, so two
//    calls whose kernels overlap on the GPU (different streams, or different host threads) race.
//    Calls issued on one stream run one after the other and are safe.
//  * Every call looks up the array's device address on the current device and context
//    (cudaGetSymbolAddress; no address is cached, so a reset device or another context gets its own
//    copy).  The first call on a device also loads this module there; make that first call before
//    any stream capture.
#include <cuda_runtime.h>
#include <cstdio>
#include "../../include/symboltz_gb300.h"
#include "sbz_los.cuh"

namespace sbz {
int capi_fail(int code, const char* msg);
}

namespace {

// File-scope scratch.  On the host `g_scratch` is only a stand-in symbol: its device address is
// obtained per device with cudaGetSymbolAddress and passed to the kernels as a plain pointer.
static __device__ __align__(256) double g_scratch[SBZ_NOALLOC_SCRATCH_DOUBLES];

// scratch layout (offsets in doubles, each region 256-byte aligned): cprime[np] | invden[np] | z[np*nl]
inline long long pad32(long long n) { return (n + 31) / 32 * 32; }

// Natural-spline Thomas factors for the points (0, k_1, ..., k_nk), shared by every multipole.
// One thread: nk is at most a few thousand.  Entries 0 and np-1, which the sweep never reads,
// are cleared because the array keeps the previous call's values.  Knots that are not positive
// and strictly increasing make every factor NaN, so the C_l come out NaN rather than wrong.
__global__ void noalloc_factors_kernel(int nk, const double* __restrict__ ks, double* __restrict__ cprime,
                                       double* __restrict__ invden) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  const int np = nk + 1;
  bool ok = true;
  double xprev = 0.0;
  for (int i = 0; i < nk; ++i) {
    const double x = ks[i];
    if (!(x > xprev) || !isfinite(x)) ok = false;
    xprev = x;
  }
  cprime[0] = 0.0; invden[0] = 0.0;
  cprime[np - 1] = 0.0; invden[np - 1] = 0.0;
  double cprev = 0.0;
  for (int i = 1; i <= np - 2; ++i) {
    const double xm = (i - 1 == 0) ? 0.0 : ks[i - 2], x0 = ks[i - 1], xp = ks[i];
    const double h0 = x0 - xm, h1 = xp - x0;
    const double inv = ok ? 1.0 / (2 * (h0 + h1) - h0 * cprev) : __longlong_as_double(0x7ff8000000000000LL);
    invden[i] = inv;
    cprev = h1 * inv;
    cprime[i] = cprev;
  }
}

// Device address of the scratch in the current device's current context, looked up on every call:
// after a device reset, or in a context other than the primary one, an address kept from an earlier
// call would point at memory that is no longer this module's.
double* scratch_for_current_device(int* err) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) { *err = 1; return nullptr; }
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) { *err = 2; return nullptr; }
  return static_cast<double*>(p);
}

}  // namespace

extern "C" int sbz_cl_integrate_noalloc(int nk, const double* d_ks, const double* d_P0, int nl, const double* d_ThA,
                                        const double* d_ThB, double* d_Cl, void* stream) {
  if (nk < 2 || nl < 1 || !d_ks || !d_P0 || !d_ThA || !d_ThB || !d_Cl)
    return sbz::capi_fail(SBZ_ERR_ARG, "sbz_cl_integrate_noalloc: bad arguments");
  const long long np = (long long)nk + 1;
  const long long need = 2 * pad32(np) + np * (long long)nl;
  if (need > (long long)SBZ_NOALLOC_SCRATCH_DOUBLES) {
    char msg[200];
    std::snprintf(msg, sizeof msg,
                  "sbz_cl_integrate_noalloc: nk=%d, nl=%d need %lld doubles of scratch; the static scratch holds %d "
                  "(2*ceil32(nk+1) + (nk+1)*nl must not exceed it)",
                  nk, nl, need, (int)SBZ_NOALLOC_SCRATCH_DOUBLES);
    return sbz::capi_fail(SBZ_ERR_ARG, msg);
  }
  int err = 0;
  double* base = scratch_for_current_device(&err);
  if (!base)
    return sbz::capi_fail(SBZ_ERR_CUDA, err == 1 ? "sbz_cl_integrate_noalloc: no current CUDA device"
                                                 : "sbz_cl_integrate_noalloc: cudaGetSymbolAddress of the scratch failed");
  double* cprime = base;
  double* invden = base + pad32(np);
  double* z = base + 2 * pad32(np);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  noalloc_factors_kernel<<<1, 32, 0, st>>>(nk, d_ks, cprime, invden);
  if (cudaGetLastError() != cudaSuccess) return sbz::capi_fail(SBZ_ERR_CUDA, "sbz_cl_integrate_noalloc: factor kernel launch");
  if (sbz::cl_launch(nk, d_ks, d_P0, nl, d_ThA, d_ThB, cprime, invden, z, d_Cl, st) != 0)
    return sbz::capi_fail(SBZ_ERR_CUDA, "sbz_cl_integrate_noalloc: C_l kernel launch");
  return SBZ_OK;
}
