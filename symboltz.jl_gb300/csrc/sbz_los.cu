// Line-of-sight kernels.
//
//   SphericalBesselCache (src/observables/angular.jl:18-26): table of j_l(x) and j_l'(x) at the
//     requested l on x = range(0, xmax, length = trunc(xmax/dx)) (+ a duplicated end point),
//     contiguous in l.  Built here by one thread per x with recurrences in l (upward where
//     l < x, Miller's downward recurrence normalised by j_0 or j_1 elsewhere).
//   cache evaluation (angular.jl:29-48): linear or cubic Hermite in x; the Hermite slopes are
//     scaled by the requested dx, as in the reference.
//   los_integrate (angular.jl:109-185): trapezoid in τ of S(τ,k) j_l(k(τ0-τ)); one block per k,
//     threads over l so every table read is a coalesced row segment; Limber branch for l >= l_limber.
//   spectrum_cmb k-integral (angular.jl:198-223): natural cubic spline through (0,0) and the
//     integrand values, integrated exactly; the tridiagonal spline system depends only on the
//     k-grid, so it is factorised once and every l runs the two sweeps.
#include <cuda_runtime.h>
#include <cstdint>
#include <cmath>
#include "sbz_los.cuh"

namespace sbz {
namespace {

__global__ void bessel_table_kernel(BesselDev J, const int* __restrict__ ls, int Lmax) {
  const int ix = blockIdx.x * blockDim.x + threadIdx.x;
  const int N = J.nx - 1;  // last row duplicates row N-1
  if (ix >= N) return;
  const double x = (ix == N - 1) ? J.xmax : ix * J.step;
  const int nl = J.nl;
  double* yrow = J.y + (size_t)ix * nl;
  double* dyrow = J.hermite ? J.dy + (size_t)ix * nl : nullptr;
  const int L = Lmax + 1;  // one above the largest l (for the derivative)
  if (x == 0.0) {
    for (int i = 0; i < nl; ++i) {
      const int l = ls[i];
      yrow[i] = (l == 0) ? 1.0 : 0.0;
      if (dyrow) dyrow[i] = (l == 1) ? 1.0 / 3.0 : 0.0;
    }
  } else {
    const double s = sin(x), c = cos(x), ix1 = 1.0 / x;
    const double j0 = s * ix1, j1 = (s * ix1 - c) * ix1;
    if (x > L) {  // upward recurrence, stable for l < x
      double jm = c * ix1, jc = j0, jn = j1;  // j_{l-1}, j_l, j_{l+1} at l = 0
      int q = 0;
      for (int l = 0; l <= Lmax && q < nl; ++l) {
        while (q < nl && ls[q] == l) {
          yrow[q] = jc;
          if (dyrow) dyrow[q] = (l == 0) ? -jn : (l * jm - (l + 1) * jn) / (2.0 * l + 1);
          ++q;
        }
        const double jnn = (2 * l + 3) * ix1 * jn - jc;
        jm = jc; jc = jn; jn = jnn;
      }
    } else {  // Miller: downward from well above max(l, x), normalised by j_0 or j_1
      const int Ls = L + 30 + (int)sqrt(40.0 * (L + 1));
      double tp = 0.0, tc = 1e-300;  // t_{l+1}, t_l at l = Ls
      int q = nl - 1;
      for (int l = Ls; l >= 1; --l) {
        const double tm = (2 * l + 1) * ix1 * tc - tp;  // t_{l-1}
        while (q >= 0 && ls[q] == l) {
          yrow[q] = tc;
          if (dyrow) dyrow[q] = (l * tm - (l + 1) * tp) / (2.0 * l + 1);
          --q;
        }
        tp = tc; tc = tm;
        if (fabs(tc) > 1e200) {  // rescale the recurrence and everything stored so far
          tp *= 1e-200; tc *= 1e-200;
          for (int r = q + 1; r < nl; ++r) { yrow[r] *= 1e-200; if (dyrow) dyrow[r] *= 1e-200; }
        }
      }
      while (q >= 0) {  // l = 0 (tc = t_0, tp = t_1)
        yrow[q] = tc;
        if (dyrow) dyrow[q] = -tp;
        --q;
      }
      const double norm = (fabs(j0) >= fabs(j1)) ? j0 / tc : j1 / tp;
      for (int r = 0; r < nl; ++r) { yrow[r] *= norm; if (dyrow) dyrow[r] *= norm; }
    }
  }
  if (ix == N - 1) {
    double* last = J.y + (size_t)N * nl;
    for (int i = 0; i < nl; ++i) last[i] = yrow[i];
    if (dyrow) { double* dl = J.dy + (size_t)N * nl; for (int i = 0; i < nl; ++i) dl[i] = dyrow[i]; }
  }
}

__device__ __forceinline__ double jl_interp(const BesselDev& J, int il, double x) {
  double w = x * J.invdx;
  const int i = (int)w;
  w -= i;
  const double ym = J.y[(size_t)i * J.nl + il], yp = J.y[(size_t)(i + 1) * J.nl + il];
  if (!J.hermite) return fma(w, yp - ym, ym);
  const double dym = J.dy[(size_t)i * J.nl + il], dyp = J.dy[(size_t)(i + 1) * J.nl + il];
  const double wm1 = w - 1.0;
  return (1 + 2 * w) * wm1 * wm1 * ym + w * w * (3 - 2 * w) * yp + w * wm1 * (wm1 * dym + w * dyp) * J.dx;
}

__global__ void bessel_eval_kernel(BesselDev J, int il, int n, const double* __restrict__ x, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = jl_interp(J, il, x[i]);
}

// One block per k; threads stride over l < il_limber.  S: [(it*nk + ik)*nsrc + s].
template <int NSRC>
__global__ void los_kernel(BesselDev J, const double* __restrict__ S, const double* __restrict__ chi,
                           const double* __restrict__ wts, int ntau, int nk, const double* __restrict__ ks,
                           int il_limber, double* __restrict__ out) {
  const int ik = blockIdx.x;
  const double k = ks[ik];
  const int nl = J.nl;
  for (int il = threadIdx.x; il < il_limber; il += blockDim.x) {
    double acc[NSRC];
#pragma unroll
    for (int s = 0; s < NSRC; ++s) acc[s] = 0;
    for (int it = 0; it < ntau; ++it) {
      const double j = jl_interp(J, il, k * chi[it]);
      const double w = wts[it];
      const double* Sp = S + ((size_t)it * nk + ik) * NSRC;
#pragma unroll
      for (int s = 0; s < NSRC; ++s) acc[s] = fma(w * __ldg(Sp + s), j, acc[s]);
    }
#pragma unroll
    for (int s = 0; s < NSRC; ++s) out[((size_t)ik * nl + il) * NSRC + s] = acc[s];
  }
  for (int il = il_limber + threadIdx.x; il < nl; il += blockDim.x)
#pragma unroll
    for (int s = 0; s < NSRC; ++s) out[((size_t)ik * nl + il) * NSRC + s] = 0;
}

// Mixed-precision line of sight: one block per k, 256 threads over l (up to 4 l per thread).
// Per chunk of 256 times the block tabulates, in FP64, what depends on (k, τ) only: the table row
// of x = k χ, the interpolation weights and w_τ S(τ, k); the l-threads then interpolate the FP32
// table and accumulate in FP32 over the chunk, adding chunk totals in FP64.
constexpr int kLosChunk = 256, kLosMaxL = 4;
template <int NSRC>
__global__ void __launch_bounds__(256) los_f32_kernel(const float2* __restrict__ tab, int nl, double invdx, double dx, int hermite,
                                                      const double* __restrict__ S, const double* __restrict__ chi,
                                                      const double* __restrict__ wts, int ntau, int nk, const double* __restrict__ ks,
                                                      int il_limber, double* __restrict__ out) {
  __shared__ int s_i[kLosChunk];
  __shared__ float4 s_w[kLosChunk];
  __shared__ float s_S[kLosChunk][NSRC];
  const int ik = blockIdx.x;
  const double k = ks[ik];
  double acc[kLosMaxL][NSRC];
#pragma unroll
  for (int m = 0; m < kLosMaxL; ++m)
#pragma unroll
    for (int s = 0; s < NSRC; ++s) acc[m][s] = 0;
  for (int t0 = 0; t0 < ntau; t0 += kLosChunk) {
    const int nt = min(kLosChunk, ntau - t0);
    __syncthreads();
    for (int t = threadIdx.x; t < nt; t += blockDim.x) {
      const int it = t0 + t;
      const double wpos = k * chi[it] * invdx;
      const int i = (int)wpos;
      const float w = (float)(wpos - i), wm1 = w - 1.0f;
      float4 ww;
      if (hermite) {
        ww.x = (1.0f + 2.0f * w) * wm1 * wm1; ww.y = w * w * (3.0f - 2.0f * w);
        ww.z = (float)(w * wm1 * wm1 * dx); ww.w = (float)(w * w * wm1 * dx);
      } else {
        ww.x = 1.0f - w; ww.y = w; ww.z = 0.0f; ww.w = 0.0f;
      }
      s_i[t] = i; s_w[t] = ww;
      const double wt = wts[it];
#pragma unroll
      for (int s = 0; s < NSRC; ++s) s_S[t][s] = (float)(wt * S[((size_t)it * nk + ik) * NSRC + s]);
    }
    __syncthreads();
#pragma unroll
    for (int m = 0; m < kLosMaxL; ++m) {
      const int il = threadIdx.x + blockDim.x * m;
      if (il < il_limber) {
        float p[NSRC];
#pragma unroll
        for (int s = 0; s < NSRC; ++s) p[s] = 0.0f;
#pragma unroll 4
        for (int t = 0; t < nt; ++t) {
          const int i = s_i[t];
          const float4 ww = s_w[t];
          const float2 a = __ldg(tab + (size_t)i * nl + il), b = __ldg(tab + (size_t)(i + 1) * nl + il);
          const float j = fmaf(ww.x, a.x, fmaf(ww.y, b.x, fmaf(ww.z, a.y, ww.w * b.y)));
#pragma unroll
          for (int s = 0; s < NSRC; ++s) p[s] = fmaf(s_S[t][s], j, p[s]);
        }
#pragma unroll
        for (int s = 0; s < NSRC; ++s) acc[m][s] += (double)p[s];
      }
    }
  }
#pragma unroll
  for (int m = 0; m < kLosMaxL; ++m) {
    const int il = threadIdx.x + blockDim.x * m;
    if (il < il_limber)
#pragma unroll
      for (int s = 0; s < NSRC; ++s) out[((size_t)ik * nl + il) * NSRC + s] = acc[m][s];
  }
  for (int il = il_limber + threadIdx.x; il < nl; il += blockDim.x)
#pragma unroll
    for (int s = 0; s < NSRC; ++s) out[((size_t)ik * nl + il) * NSRC + s] = 0;
}

__global__ void bessel_f32_kernel(BesselDev J) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)J.nx * J.nl) return;
  J.yf2[t] = make_float2((float)J.y[t], J.dy ? (float)J.dy[t] : 0.0f);
}

// C_l as a weighted sum over k: one block per (pair, l), FP64 throughout.
__global__ void __launch_bounds__(256) cl_dot_kernel(int nk, const double* __restrict__ g, int nl, int ns,
                                                     const double* __restrict__ Th, const int* __restrict__ pa,
                                                     const int* __restrict__ pb, double* __restrict__ Cl) {
  const int il = blockIdx.x % nl, q = blockIdx.x / nl;
  const int A = pa[q], B = pb[q];
  double sum = 0;
  for (int i = threadIdx.x; i < nk; i += blockDim.x) {
    const size_t o = ((size_t)i * nl + il) * ns;
    sum = fma(g[i] * Th[o + A], Th[o + B], sum);
  }
  __shared__ double red[8];
#pragma unroll
  for (int o = 16; o; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sum;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
    Cl[blockIdx.x] = tot;
  }
}

// Limber approximation (src/observables/angular.jl:154-178); one thread per (k, l >= l_limber).
__global__ void limber_kernel(const int* __restrict__ ls, int nl, int il_limber, int nsrc, const double* __restrict__ S,
                              const double* __restrict__ taus, const double* __restrict__ chi, int ntau, int nk,
                              const double* __restrict__ ks, double* __restrict__ out) {
  const int nlim = nl - il_limber;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nk * nlim) return;
  const int ik = t / nlim, il = il_limber + t % nlim;
  const double k = ks[ik], l = ls[il];
  const double x = (l + 0.5) / k;
  const double tau0 = taus[ntau - 1];
  for (int s = 0; s < nsrc; ++s) out[((size_t)ik * nl + il) * nsrc + s] = 0;
  if (!(x <= chi[0])) return;
  // first index with taus[i] >= tau0 - x
  int lo = 0, hi = ntau;
  const double target = tau0 - x;
  while (lo < hi) { const int mid = (lo + hi) >> 1; if (taus[mid] < target) lo = mid + 1; else hi = mid; }
  const int im = lo;
  if (im == 0) return;
  const int ip = im - 1;
  const double chim = chi[im], chip = chi[ip], dchi = chip - chim;
  for (int s = 0; s < nsrc; ++s) {
    auto Sv = [&](int i) { return S[((size_t)i * nk + ik) * nsrc + s]; };
    const double Sm = Sv(im), Sp = Sv(ip);
    const double dSm = (im <= ntau - 2) ? (Sv(im + 1) - Sp) / (chi[im + 1] - chip) : (Sp - Sm) / dchi;
    const double dSp = (ip >= 1) ? (Sm - Sv(im - 2)) / (chim - chi[im - 2]) : (Sp - Sm) / dchi;
    const double u = (x - chim) / dchi, u2 = u * u, u3 = u2 * u;
    const double Sx = (2 * u3 - 3 * u2 + 1) * Sm + (u3 - 2 * u2 + u) * dchi * dSm + (-2 * u3 + 3 * u2) * Sp + (u3 - u2) * dchi * dSp;
    out[((size_t)ik * nl + il) * nsrc + s] = sqrt(M_PI / (2 * l + 1)) * Sx / k;
  }
}

// C_l: natural cubic spline (z0 = zN = 0) through (0,0),(k_i, y_i); factors of the interior
// tridiagonal system (shared by all l) are precomputed: cprime[i], inv_den[i].
__global__ void cl_kernel(int nk, const double* __restrict__ ks, const double* __restrict__ P0, int nl,
                          const double* __restrict__ ThA, const double* __restrict__ ThB,
                          const double* __restrict__ cprime, const double* __restrict__ invden,
                          double* __restrict__ zbuf, double* __restrict__ Cl) {
  const int il = blockIdx.x * blockDim.x + threadIdx.x;
  if (il >= nl) return;
  const int np = nk + 1;  // points incl. (0, 0)
  auto X = [&](int i) { return i == 0 ? 0.0 : ks[i - 1]; };
  auto Y = [&](int i) { return i == 0 ? 0.0 : (2.0 / M_PI) * ks[i - 1] * ks[i - 1] * P0[i - 1] * ThA[(size_t)(i - 1) * nl + il] * ThB[(size_t)(i - 1) * nl + il]; };
  double* z = zbuf + (size_t)il;  // strided by nl: z[i * nl]
  // forward sweep on interior rows i = 1..np-2 (Thomas), d' stored in z
  double yprev = Y(0), ycur = Y(1);
  double dprev = 0;
  for (int i = 1; i <= np - 2; ++i) {
    const double ynext = Y(i + 1);
    const double h0 = X(i) - X(i - 1), h1 = X(i + 1) - X(i);
    const double rhs = 6 * ((ynext - ycur) / h1 - (ycur - yprev) / h0);
    const double d = (rhs - h0 * dprev) * invden[i];
    z[(size_t)i * nl] = d;
    dprev = d;
    yprev = ycur; ycur = ynext;
  }
  // back substitution; integrate on the fly
  double znext = 0, sum = 0;  // z_{np-1} = 0
  double ynext = Y(np - 1);
  for (int i = np - 2; i >= 0; --i) {
    const double zi = (i >= 1) ? z[(size_t)i * nl] - cprime[i] * znext : 0.0;
    const double yi = Y(i);
    const double h = X(i + 1) - X(i);
    sum += h * (yi + ynext) * 0.5 - h * h * h * (zi + znext) / 24.0;
    znext = zi; ynext = yi;
  }
  Cl[il] = sum;
}

// ---- source k-interpolation (src/observables/fourier.jl:227-247, 464-547) --------------------
// Coarse sources Sc[(i*ntau + j)*3 + src[s]] (perturbation-kernel layout) -> fine
// Sf[(j*nf + f)*ns + s] (line-of-sight layout).  Columns c = j*ns + s.
// Natural cubic spline in y = f(k): the tridiagonal factors depend only on the coarse y grid.
__global__ void kinterp_spline_z(int nc, int ntau, int ns, const int* __restrict__ src, const double* __restrict__ Sc,
                                 const double* __restrict__ y, const double* __restrict__ cprime,
                                 const double* __restrict__ invden, double* __restrict__ z) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ntau * ns) return;
  const int j = col / ns, s = src[col % ns];
  const int ncol = ntau * ns;
  auto V = [&](int i) { return Sc[((size_t)i * ntau + j) * 3 + s]; };
  double vprev = V(0), vcur = V(1), dprev = 0;
  z[col] = 0;
  for (int i = 1; i <= nc - 2; ++i) {
    const double vnext = V(i + 1);
    const double h0 = y[i] - y[i - 1], h1 = y[i + 1] - y[i];
    const double d = (6 * ((vnext - vcur) / h1 - (vcur - vprev) / h0) - h0 * dprev) * invden[i];
    z[(size_t)i * ncol + col] = d;
    dprev = d; vprev = vcur; vcur = vnext;
  }
  double znext = 0;
  z[(size_t)(nc - 1) * ncol + col] = 0;
  for (int i = nc - 2; i >= 1; --i) {
    const double zi = z[(size_t)i * ncol + col] - cprime[i] * znext;
    z[(size_t)i * ncol + col] = zi;
    znext = zi;
  }
}

__global__ void kinterp_spline_eval(int nc, int ntau, int ns, int nf, const int* __restrict__ src, const double* __restrict__ Sc,
                                    const double* __restrict__ y, const double* __restrict__ yf, const int* __restrict__ iv,
                                    const double* __restrict__ z, double* __restrict__ Sf) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t total = (size_t)ntau * nf * ns;
  if (t >= total) return;
  const int s = (int)(t % ns), f = (int)((t / ns) % nf), j = (int)(t / ((size_t)ns * nf));
  const int ncol = ntau * ns, col = j * ns + s;
  const int i = iv[f];
  const double h = y[i + 1] - y[i], a = y[i + 1] - yf[f], b = yf[f] - y[i];
  const double v0 = Sc[((size_t)i * ntau + j) * 3 + src[s]], v1 = Sc[((size_t)(i + 1) * ntau + j) * 3 + src[s]];
  const double z0 = z[(size_t)i * ncol + col], z1 = z[(size_t)(i + 1) * ncol + col];
  Sf[t] = z0 * a * a * a / (6 * h) + z1 * b * b * b / (6 * h) + (v1 / h - z1 * h / 6) * b + (v0 / h - z0 * h / 6) * a;
}

// Barycentric interpolation (Chebyshev points): Sf = Σ_c M[f][c] Sc[c], M built on the host.
__global__ void kinterp_bary(int nc, int ntau, int ns, int nf, const int* __restrict__ src, const double* __restrict__ Sc,
                             const double* __restrict__ Mw, double* __restrict__ Sf) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t total = (size_t)ntau * nf * ns;
  if (t >= total) return;
  const int s = (int)(t % ns), f = (int)((t / ns) % nf), j = (int)(t / ((size_t)ns * nf));
  const double* m = Mw + (size_t)f * nc;
  double acc = 0;
  for (int c = 0; c < nc; ++c) acc = fma(m[c], Sc[((size_t)c * ntau + j) * 3 + src[s]], acc);
  Sf[t] = acc;
}

// Θ scaling after the line-of-sight integral (angular.jl:301-306): T /= k; E *= √((l+2)!/(l-2)!)/k².
__global__ void theta_scale(int nk, int nl, int ns, const double* __restrict__ ks, const int* __restrict__ ls,
                            int sT, int sE, double* __restrict__ Th) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)nk * nl) return;
  const int ik = (int)(t / nl), il = (int)(t % nl);
  const double k = ks[ik], l = ls[il];
  if (sT >= 0) Th[t * ns + sT] /= k;
  if (sE >= 0) Th[t * ns + sE] *= sqrt((l + 2) * (l + 1) * l * (l - 1)) / (k * k);
}

}  // namespace

int kinterp_spline_launch(int nc, int ntau, int ns, int nf, const int* d_src, const double* d_Sc, const double* d_y,
                          const double* d_yf, const int* d_iv, const double* d_cprime, const double* d_invden, double* d_z,
                          double* d_Sf, cudaStream_t st) {
  const int ncol = ntau * ns;
  kinterp_spline_z<<<(ncol + 127) / 128, 128, 0, st>>>(nc, ntau, ns, d_src, d_Sc, d_y, d_cprime, d_invden, d_z);
  const size_t total = (size_t)ntau * nf * ns;
  kinterp_spline_eval<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(nc, ntau, ns, nf, d_src, d_Sc, d_y, d_yf, d_iv, d_z, d_Sf);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int kinterp_bary_launch(int nc, int ntau, int ns, int nf, const int* d_src, const double* d_Sc, const double* d_M, double* d_Sf,
                        cudaStream_t st) {
  const size_t total = (size_t)ntau * nf * ns;
  kinterp_bary<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(nc, ntau, ns, nf, d_src, d_Sc, d_M, d_Sf);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int theta_scale_launch(int nk, int nl, int ns, const double* d_ks, const int* d_ls, int sT, int sE, double* d_Th, cudaStream_t st) {
  const size_t total = (size_t)nk * nl;
  theta_scale<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(nk, nl, ns, d_ks, d_ls, sT, sE, d_Th);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int bessel_build(BesselDev& J, const int* d_ls, int Lmax, cudaStream_t st) {
  const int N = J.nx - 1;
  bessel_table_kernel<<<(N + 127) / 128, 128, 0, st>>>(J, d_ls, Lmax);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int bessel_f32_build(const BesselDev& J, cudaStream_t st) {
  const size_t total = (size_t)J.nx * J.nl;
  bessel_f32_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(J);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int los_f32_launch(const BesselDev& J, const int* d_ls, int nsrc, const double* d_S, const double* d_taus, const double* d_chi,
                   const double* d_w, int ntau, int nk, const double* d_ks, int il_limber, double* d_out, cudaStream_t st) {
  if (!J.yf2 || il_limber > 256 * kLosMaxL || nk <= 0) return -1;
  switch (nsrc) {
    case 1: los_f32_kernel<1><<<nk, 256, 0, st>>>(J.yf2, J.nl, J.invdx, J.dx, J.hermite, d_S, d_chi, d_w, ntau, nk, d_ks, il_limber, d_out); break;
    case 2: los_f32_kernel<2><<<nk, 256, 0, st>>>(J.yf2, J.nl, J.invdx, J.dx, J.hermite, d_S, d_chi, d_w, ntau, nk, d_ks, il_limber, d_out); break;
    case 3: los_f32_kernel<3><<<nk, 256, 0, st>>>(J.yf2, J.nl, J.invdx, J.dx, J.hermite, d_S, d_chi, d_w, ntau, nk, d_ks, il_limber, d_out); break;
    default: return -1;
  }
  const int nlim = J.nl - il_limber;
  if (nlim > 0) {
    const int tot = nk * nlim;
    limber_kernel<<<(tot + 127) / 128, 128, 0, st>>>(d_ls, J.nl, il_limber, nsrc, d_S, d_taus, d_chi, ntau, nk, d_ks, d_out);
  }
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int cl_dot_launch(int nk, const double* d_g, int nl, int ns, const double* d_Th, int npair, const int* d_pa, const int* d_pb,
                  double* d_Cl, cudaStream_t st) {
  cl_dot_kernel<<<nl * npair, 256, 0, st>>>(nk, d_g, nl, ns, d_Th, d_pa, d_pb, d_Cl);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int bessel_eval(const BesselDev& J, int il, int n, const double* d_x, double* d_out, cudaStream_t st) {
  bessel_eval_kernel<<<(n + 255) / 256, 256, 0, st>>>(J, il, n, d_x, d_out);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int los_launch(const BesselDev& J, const int* d_ls, int nsrc, const double* d_S, const double* d_taus,
               const double* d_chi, const double* d_w, int ntau, int nk, const double* d_ks, int il_limber,
               double* d_out, cudaStream_t st) {
  const int threads = 128;
  if (nk > 0) {
    switch (nsrc) {
      case 1: los_kernel<1><<<nk, threads, 0, st>>>(J, d_S, d_chi, d_w, ntau, nk, d_ks, il_limber, d_out); break;
      case 2: los_kernel<2><<<nk, threads, 0, st>>>(J, d_S, d_chi, d_w, ntau, nk, d_ks, il_limber, d_out); break;
      case 3: los_kernel<3><<<nk, threads, 0, st>>>(J, d_S, d_chi, d_w, ntau, nk, d_ks, il_limber, d_out); break;
      default: return -1;
    }
  }
  const int nlim = J.nl - il_limber;
  if (nlim > 0 && nk > 0) {
    const int tot = nk * nlim;
    limber_kernel<<<(tot + 127) / 128, 128, 0, st>>>(d_ls, J.nl, il_limber, nsrc, d_S, d_taus, d_chi, ntau, nk, d_ks, d_out);
  }
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int cl_launch(int nk, const double* d_ks, const double* d_P0, int nl, const double* d_ThA, const double* d_ThB,
              const double* d_cprime, const double* d_invden, double* d_zbuf, double* d_Cl, cudaStream_t st) {
  cl_kernel<<<(nl + 127) / 128, 128, 0, st>>>(nk, d_ks, d_P0, nl, d_ThA, d_ThB, d_cprime, d_invden, d_zbuf, d_Cl);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

}  // namespace sbz
