#pragma once
// Perturbation solver kernel (implementation; instantiated in sbz_pt_f32.cu / sbz_pt_f64.cu): one warp integrates one (cosmology, k) mode.
//
// Replaces the per-k loop of solvept (src/solve.jl:543-569) and the Rodas5P + KLU inner solver
// it calls (src/solve.jl:327-341).  Integrator: Hairer-Wanner RODAS (Rosenbrock, order 4(3),
// stiffly accurate) in transformed form
//   (1/(hγ) - J) U_i = f(t+c_i h, y + Σ A_ij U_j) + Σ (C_ij/h) U_j + h d_i ∂f/∂τ,
//   y1 = y + Σ A_5j U_j + U_5 + U_6, error estimate U_6,
// with the error norm, PI step-size control and Hermite dense output of OrdinaryDiffEq-style
// integrators.  The perturbation system is linear, u' = J(τ) u, so "f" and "J·x" are one
// operator; its rows are described in sbz_layout.hpp.
//
// Stage solves exploit the structure of M = 1/(hγ) - B (J = B + c_Φ̇ ∇Φ̇ᵀ + c_Ψ ∇Ψᵀ):
//   * the free-streaming hierarchies are tridiagonal chains, eliminated from their truncation
//     end by one lane each (all chains in parallel, no pivoting needed: pivots stay ≥ 1/(hγ));
//   * photon-baryon rows δb, θb, F0-2, G0-2 form a dense 8x8 head (LU with partial pivoting);
//   * CDM and Φ are 2x2/1x1 triangular blocks;
//   * the two metric couplings are added back with a rank-2 Sherman-Morrison-Woodbury update.
// ST = double: all-FP64 solve.  ST = float: FP32 factorisation and solves with FP64 iterative
// refinement against the FP64 operator (residuals, state, error norm and step control in FP64).
//
// Lanes own components i = lane + 32 s.  Warp-uniform control flow; every wait is a __syncwarp.
// Loops are bounded by opts.maxiters and a step-size floor, so a mode that cannot finish sets a
// status code and the warp moves on.
#include <cuda_runtime.h>
#include <cstdint>
#include "sbz_layout.hpp"
#include "sbz_pt.cuh"

namespace sbz {
namespace ptk {

constexpr unsigned FULL = 0xffffffffu;

namespace rw {
constexpr double gam = 0.25;
constexpr double c2 = 0.386, c3 = 0.21, c4 = 0.63;
constexpr double d1 = 0.25, d2 = -0.1043, d3 = 0.1035, d4 = -0.0362;
constexpr double A21 = 1.544, A31 = 0.9466785280815826, A32 = 0.2557011698983284;
constexpr double A41 = 3.314825187068521, A42 = 2.896124015972201, A43 = 0.9986419139977817;
constexpr double A51 = 1.221224509226641, A52 = 6.019134481288629, A53 = 12.53708332932087, A54 = -0.6878860361058950;
constexpr double C21 = -5.6688, C31 = -2.430093356833875, C32 = -0.2063599157091915;
constexpr double C41 = -0.1073529058151375, C42 = -9.594562251023355, C43 = -20.47028614809616;
constexpr double C51 = 7.496443313967647, C52 = -10.24680431464352, C53 = -33.99990352819905, C54 = 11.70890893206160;
constexpr double C61 = 8.083246795921522, C62 = -7.981132988064893, C63 = -31.52159432874371, C64 = 16.31930543123136, C65 = -6.058818238834054;
}  // namespace rw

constexpr int kWF = 2 * kMaxFun;  // functional weights per set: Ψ terms then δρ terms

static_assert(sizeof(ModelDesc) % 4 == 0 && sizeof(CompDesc) % 4 == 0, "word copies");

template <int NS, typename ST>
struct WarpMem {
  static constexpr int NM = 32 * NS;
  double x[NM + 1];   // operator input; x[n] stays 0
  double f[NM + 1];   // J y at output points; f[n] stays 0
  ST r[NM + 1];       // structured-solve right-hand side / solution
  ST dinv[NM], sub[NM], sup[NM];
  ST Z1[NM], Z2[NM];
  ST H[64];
  ST hsup[2], hcorr[2];
  int piv[8];
  double cvJ[kNCV], cvdJ[kNCV], wJ[kWF], wdJ[kWF];   // coefficients at the step start
  double cvS[kNCV], cvdS[kNCV], wS[kWF], wdS[kWF];   // coefficients at a stage / output time
  double B[B_COUNT], dB[B_COUNT];
  double src[4];      // e^{-κ}, κ̈, κ⃛ at an output time
};

struct Coef {  // pointers to one coefficient set in shared memory
  double *cv, *cvd, *w, *wd;
};

__device__ __forceinline__ double bcast(double v, int src) { return __shfl_sync(FULL, v, src); }

// ------------------------------------------------------------------------------------------
// τ-dependent coefficients (values and, with deriv, d/dτ) at time tau.
// source = true: also fetch e^{-κ}, κ̈, κ⃛ and use the Taylor-mode κ̈ as dκ̇/dτ (the line-of-sight
// sources differentiate the background along its ODE, src/models/cosmologies.jl:99-105).
template <int NS, typename ST>
__device__ void coef_eval(WarpMem<NS, ST>& W, const Coef& C, const CosmoDesc* __restrict__ cd,
                          const double* __restrict__ tab, int nexpr, int nx, double k, double tau,
                          bool deriv, bool source) {
  const int lane = threadIdx.x & 31;
  const int ntab = cd->ntab;
  int g = (int)((__logf((float)tau) - (float)cd->lnt0) * (float)cd->idlnt);
  g = max(0, min(g, ntab - 2));
  const double* nd = tab + (size_t)g * kNodeStride;
  if (tau < nd[0] && g > 0) { --g; nd -= kNodeStride; }
  else if (tau > nd[kNodeStride] && g < ntab - 2) { ++g; nd += kNodeStride; }
  // Hermite pairs q = 0..6 on lanes 0..6: a, ℋ, κ̇, c_s², e^{-κ}, κ̈, κ⃛
  double v = 0, dv = 0;
  {
    const int q = lane < 7 ? lane : 0;
    const double t0 = nd[0], ih = nd[1], h = nd[kNodeStride] - t0;
    const double s = (tau - t0) * ih, s2 = s * s, s3 = s2 * s;
    const double v0 = nd[2 + 2 * q], d0 = nd[3 + 2 * q], v1 = nd[kNodeStride + 2 + 2 * q], d1 = nd[kNodeStride + 3 + 2 * q];
    v = (2 * s3 - 3 * s2 + 1) * v0 + (s3 - 2 * s2 + s) * h * d0 + (3 * s2 - 2 * s3) * v1 + (s3 - s2) * h * d1;
    dv = ((6 * s2 - 6 * s) * v0 + (6 * s - 6 * s2) * v1) * ih + (3 * s2 - 4 * s + 1) * d0 + (3 * s2 - 2 * s) * d1;
  }
  const double a = bcast(v, 0), da = bcast(dv, 0);
  const double Hc = bcast(v, 1), dHc = bcast(dv, 1);
  const double kd = bcast(v, 2);
  double dkd = bcast(dv, 2);
  const double cs2 = bcast(v, 3), dcs2 = bcast(dv, 3);
  if (source) {
    const double ek = bcast(v, 4), kdd = bcast(v, 5), kddd = bcast(v, 6);
    dkd = kdd;
    if (lane == 0) { W.src[0] = ek; W.src[1] = kdd; W.src[2] = kddd; }
  }
  // reciprocals and momentum-bin energies, one value per lane (lane 0: a, 1: τ, 2: ℋ, 3+j: E_j)
  const int jb = (lane >= 3 ? lane - 3 : 0) & (kMaxNx - 1);
  const double xj = cd->xq[jb];
  const double y0a = cd->y0 * a;
  const double E = sqrt(xj * xj + y0a * y0a);
  const double dE = (E > 0) ? cd->y0 * y0a * da / E : 0.0;
  const double rv = lane == 0 ? a : lane == 1 ? tau : lane == 2 ? Hc : E;
  const double drv = lane == 0 ? da : lane == 1 ? 1.0 : lane == 2 ? dHc : dE;
  const double inv = 1.0 / rv;
  const double dinv = -drv * inv * inv;
  if (lane >= 3 && lane - 3 < nx) {
    const int j = lane - 3;
    const double ixj = 1.0 / xj;
    W.B[B_Q + j] = xj * inv; W.B[B_IQ + j] = E * ixj; W.B[B_E + j] = E; W.B[B_IE + j] = inv;
    W.dB[B_Q + j] = xj * dinv; W.dB[B_IQ + j] = dE * ixj; W.dB[B_E + j] = dE; W.dB[B_IE + j] = dinv;
  }
  const double ia = bcast(inv, 0), dia = bcast(dinv, 0);
  const double itau = bcast(inv, 1), ditau = bcast(dinv, 1);
  const double iH = bcast(inv, 2), diH = bcast(dinv, 2);
  if (lane == 0) {
    W.B[B_ONE] = 1; W.B[B_K] = k; W.B[B_K2] = k * k; W.B[B_IK] = 1 / k; W.B[B_IK2] = 1 / (k * k);
    W.B[B_KD] = kd; W.B[B_H] = Hc; W.B[B_CS2] = cs2; W.B[B_IA] = ia; W.B[B_IA2] = ia * ia;
    W.B[B_R] = cd->R0 * ia; W.B[B_IH] = iH; W.B[B_ITAU] = itau;
    W.dB[B_ONE] = 0; W.dB[B_K] = 0; W.dB[B_K2] = 0; W.dB[B_IK] = 0; W.dB[B_IK2] = 0;
    W.dB[B_KD] = dkd; W.dB[B_H] = dHc; W.dB[B_CS2] = dcs2; W.dB[B_IA] = dia; W.dB[B_IA2] = 2 * ia * dia;
    W.dB[B_R] = cd->R0 * dia; W.dB[B_IH] = diH; W.dB[B_ITAU] = ditau;
  }
  __syncwarp();
  for (int e = lane; e < nexpr; e += 32) {
    const CoefExpr& X = cd->expr[e];
    const double p0 = W.B[X.b[0]], p1 = W.B[X.b[1]], p2 = W.B[X.b[2]];
    const double q0 = W.B[X.b[3]], q1 = W.B[X.b[4]], q2 = W.B[X.b[5]];
    const double val = X.K1 * (p0 * p1 * p2) + X.K2 * (q0 * q1 * q2);
    double dval = 0;
    if (deriv) {
      const double dp0 = W.dB[X.b[0]], dp1 = W.dB[X.b[1]], dp2 = W.dB[X.b[2]];
      const double dq0 = W.dB[X.b[3]], dq1 = W.dB[X.b[4]], dq2 = W.dB[X.b[5]];
      dval = X.K1 * (dp0 * p1 * p2 + p0 * dp1 * p2 + p0 * p1 * dp2) + X.K2 * (dq0 * q1 * q2 + q0 * dq1 * q2 + q0 * q1 * dq2);
    }
    const int d = X.dest;
    if (d < kNCV) { C.cv[d] = val; C.cvd[d] = dval; }
    else { C.w[d - kNCV] = val; C.wd[d - kNCV] = dval; }
  }
  __syncwarp();
}

// Metric functionals of a shared-memory vector v: Ψ(v) and the δρ sum; Φ̇ = PA·ρ + PB·v_Φ + (-ℋ)Ψ.
template <typename T>
__device__ __forceinline__ void functionals(const T* v, const double* w, const ModelDesc& M, double& psi, double& rho) {
  const int lane = threadIdx.x & 31;
  double t = 0;
  if (lane < M.npsi) t = w[lane] * (double)v[M.psiComp[lane]];
  else if (lane >= kMaxFun && lane - kMaxFun < M.nrho) t = w[lane] * (double)v[M.rhoComp[lane - kMaxFun]];
#pragma unroll
  for (int o = 8; o; o >>= 1) t += __shfl_xor_sync(FULL, t, o);
  psi = __shfl_sync(FULL, t, 0);
  rho = __shfl_sync(FULL, t, 16);
}

__device__ __forceinline__ double phidot(const double* cv, double rho, double xphi, double psi) {
  return cv[CV_PA] * rho + cv[CV_PB] * xphi + cv[CV_MH] * psi;
}

// out = J(τ) x for the lane's components (x in shared memory, x[n] == 0).
template <int NS, typename ST>
__device__ __forceinline__ void matvec(const WarpMem<NS, ST>& W, const double* x, const double* cv, const double* w,
                                       const CompDesc* __restrict__ comps, const ModelDesc& M, double k,
                                       double (&out)[NS], double* phid_out = nullptr, double* psi_out = nullptr) {
  const int lane = threadIdx.x & 31;
  double psi, rho;
  functionals(x, w, M, psi, rho);
  const double phd = phidot(cv, rho, x[0], psi);
  if (phid_out) *phid_out = phd;
  if (psi_out) *psi_out = psi;
  const double k34 = 0.75 * k;
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    const int i = lane + 32 * s;
    double o = 0;
    if (i < M.n) {
      const CompDesc& D = comps[i];
      o = cv[D.sp] * (D.A * x[D.ip] + D.C * x[D.inx]) + (cv[D.dg] + cv[D.tr]) * x[i] + cv[D.phid] * phd + cv[D.psid] * psi;
      if (s == 0) o += cv[D.e0] * x[D.e0c] + cv[D.e1] * x[D.e1c] + cv[D.e2] * x[D.e2c] + cv[D.dx] * (x[D.dxa] - k34 * x[D.dxb]);
    }
    out[s] = o;
  }
}

// out = (dJ/dτ) x
template <int NS, typename ST>
__device__ __forceinline__ void matvec_dtau(const WarpMem<NS, ST>& W, const double* x, const Coef& C,
                                            const CompDesc* __restrict__ comps, const ModelDesc& M, double k,
                                            double (&out)[NS], double* dpsi_out = nullptr) {
  const int lane = threadIdx.x & 31;
  double psi, rho, dpsi, drho;
  functionals(x, C.w, M, psi, rho);
  functionals(x, C.wd, M, dpsi, drho);
  const double* cv = C.cv; const double* cvd = C.cvd;
  const double phd = phidot(cv, rho, x[0], psi);
  const double dphd = cvd[CV_PA] * rho + cv[CV_PA] * drho + cvd[CV_PB] * x[0] + cvd[CV_MH] * psi + cv[CV_MH] * dpsi;
  if (dpsi_out) *dpsi_out = dpsi;
  const double k34 = 0.75 * k;
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    const int i = lane + 32 * s;
    double o = 0;
    if (i < M.n) {
      const CompDesc& D = comps[i];
      o = cvd[D.sp] * (D.A * x[D.ip] + D.C * x[D.inx]) + (cvd[D.dg] + cvd[D.tr]) * x[i] + cvd[D.phid] * phd +
          cv[D.phid] * dphd + cvd[D.psid] * psi + cv[D.psid] * dpsi;
      if (s == 0) o += cvd[D.e0] * x[D.e0c] + cvd[D.e1] * x[D.e1c] + cvd[D.e2] * x[D.e2c] + cvd[D.dx] * (x[D.dxa] - k34 * x[D.dxb]);
    }
    out[s] = o;
  }
}

// ------------------------------------------------------------------------------------------
// structured factorisation of M = s I - B and its solves
__device__ __forceinline__ int head_local(int i) { return (i >= 3 && i <= 10) ? i - 3 : -1; }

template <int NS, typename ST>
__device__ void solve_M(WarpMem<NS, ST>& W, const ModelDesc& M, ST is, ST ihc) {
  const int lane = threadIdx.x & 31;
  if (lane < M.nchain) {  // forward elimination, truncation end first
    const int first = M.chFirst[lane], last = M.chLast[lane];
    ST carry = W.r[last];
    for (int i = last - 1; i >= first; --i) {
      carry = W.r[i] - W.sup[i] * carry * W.dinv[i + 1];
      W.r[i] = carry;
    }
    const int at = M.chAttach[lane];
    if (at >= 0) W.r[at] -= W.hsup[lane] * W.r[first] * W.dinv[first];
  }
  __syncwarp();
  if (lane == 0) {  // 8x8 head: LU solve
    ST b[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) b[j] = W.r[3 + j];
#pragma unroll
    for (int j = 0; j < 8; ++j) { const int p = W.piv[j]; if (p != j) { ST t = b[j]; b[j] = b[p]; b[p] = t; } }
#pragma unroll
    for (int i = 1; i < 8; ++i) {
      ST s = b[i];
#pragma unroll
      for (int j = 0; j < i; ++j) s -= W.H[i * 8 + j] * b[j];
      b[i] = s;
    }
#pragma unroll
    for (int i = 7; i >= 0; --i) {
      ST s = b[i];
#pragma unroll
      for (int j = i + 1; j < 8; ++j) s -= W.H[i * 8 + j] * b[j];
      b[i] = s * W.H[i * 8 + i];  // diagonal holds the reciprocal pivot
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) W.r[3 + j] = b[j];
  } else if (lane == 1) {  // CDM: [[s, 1], [0, s+ℋ]]
    const ST zt = W.r[2] * ihc;
    W.r[2] = zt;
    W.r[1] = (W.r[1] - zt) * is;
  } else if (lane == 2) {
    W.r[0] = W.r[0] * is;
  }
  __syncwarp();
  if (lane < M.nchain) {  // back substitution away from the head
    const int first = M.chFirst[lane], last = M.chLast[lane], at = M.chAttach[lane];
    ST zp = at >= 0 ? W.r[at] : ST(0);
    for (int i = first; i <= last; ++i) {
      zp = (W.r[i] - W.sub[i] * zp) * W.dinv[i];
      W.r[i] = zp;
    }
  }
  __syncwarp();
}

template <int NS, typename ST>
struct Factor {
  ST is, ihc;
  double S00, S01, S10, S11;  // inverse of I - Vᵀ M⁻¹ U
};

template <int NS, typename ST>
__device__ void factorize(WarpMem<NS, ST>& W, Factor<NS, ST>& F, const double* cv, const double* w,
                          const CompDesc* __restrict__ comps, const ModelDesc& M, double k, double s) {
  const int lane = threadIdx.x & 31;
  const double k34 = 0.75 * k;
  if (lane < M.nchain) {
    const int first = M.chFirst[lane], last = M.chLast[lane], at = M.chAttach[lane];
    ST dnext = 0, subnext = 0;
    for (int i = last; i >= first; --i) {
      const CompDesc& D = comps[i];
      const double spv = cv[D.sp];
      double mii = s - (cv[D.dg] + cv[D.tr]);
      const ST sup = (ST)(-spv * D.C), sub = (ST)(-spv * D.A);
      if (i < last) mii -= (double)(sup * subnext * dnext);
      const ST di = (ST)(1.0 / mii);
      W.dinv[i] = di; W.sup[i] = sup; W.sub[i] = sub;
      dnext = di; subnext = sub;
    }
    if (at >= 0) {
      const CompDesc& D = comps[at];
      const ST hs = (ST)(-cv[D.sp] * D.C);  // coefficient of x[first] in the head row
      W.hsup[lane] = hs;
      W.hcorr[lane] = hs * subnext * dnext;
    }
  }
  __syncwarp();
  if (lane < 8) {  // assemble head row 3+lane
    const int r = 3 + lane;
    const CompDesc& D = comps[r];
    double row[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) row[j] = 0;
    row[lane] += s - (cv[D.dg] + cv[D.tr]);
    const double spv = cv[D.sp];
    int c;
    if ((c = head_local(D.ip)) >= 0) row[c] -= spv * D.A;
    if ((c = head_local(D.inx)) >= 0) row[c] -= spv * D.C;
    if ((c = head_local(D.e0c)) >= 0) row[c] -= cv[D.e0];
    if ((c = head_local(D.e1c)) >= 0) row[c] -= cv[D.e1];
    if ((c = head_local(D.e2c)) >= 0) row[c] -= cv[D.e2];
    if ((c = head_local(D.dxa)) >= 0) row[c] -= cv[D.dx];
    if ((c = head_local(D.dxb)) >= 0) row[c] += k34 * cv[D.dx];
    if (r == 7) row[4] -= (double)W.hcorr[0];   // F2 (Schur complement of the F tail)
    if (r == 10) row[7] -= (double)W.hcorr[1];  // G2 (G tail)
#pragma unroll
    for (int j = 0; j < 8; ++j) W.H[lane * 8 + j] = (ST)row[j];
  }
  __syncwarp();
  if (lane == 0) {  // LU with partial pivoting; store reciprocal pivots on the diagonal
    for (int kk = 0; kk < 8; ++kk) {
      int p = kk; ST mx = fabs(W.H[kk * 8 + kk]);
      for (int i = kk + 1; i < 8; ++i) { const ST v = fabs(W.H[i * 8 + kk]); if (v > mx) { mx = v; p = i; } }
      W.piv[kk] = p;
      if (p != kk) for (int j = 0; j < 8; ++j) { const ST t = W.H[kk * 8 + j]; W.H[kk * 8 + j] = W.H[p * 8 + j]; W.H[p * 8 + j] = t; }
      const ST ip = ST(1) / W.H[kk * 8 + kk];
      W.H[kk * 8 + kk] = ip;
      for (int i = kk + 1; i < 8; ++i) {
        const ST l = W.H[i * 8 + kk] * ip;
        W.H[i * 8 + kk] = l;
        for (int j = kk + 1; j < 8; ++j) W.H[i * 8 + j] -= l * W.H[kk * 8 + j];
      }
    }
  }
  F.is = (ST)(1.0 / s);
  F.ihc = (ST)(1.0 / (s - cv[CV_MH]));
  __syncwarp();
  // rank-2 correction: Z1 = M⁻¹ c_Φ̇, Z2 = M⁻¹ c_Ψ
  double psi1, rho1, psi2, rho2;
  for (int pass = 0; pass < 2; ++pass) {
#pragma unroll
    for (int sl = 0; sl < NS; ++sl) {
      const int i = lane + 32 * sl;
      if (i < M.n) W.r[i] = (ST)cv[pass == 0 ? comps[i].phid : comps[i].psid];
    }
    __syncwarp();
    solve_M(W, M, F.is, F.ihc);
#pragma unroll
    for (int sl = 0; sl < NS; ++sl) {
      const int i = lane + 32 * sl;
      if (i < M.n) (pass == 0 ? W.Z1 : W.Z2)[i] = W.r[i];
    }
    if (pass == 0) functionals(W.r, w, M, psi1, rho1);
    else functionals(W.r, w, M, psi2, rho2);
    __syncwarp();
  }
  const double p1 = phidot(cv, rho1, (double)W.Z1[0], psi1), p2 = phidot(cv, rho2, (double)W.Z2[0], psi2);
  const double a = 1 - p1, b = -p2, c = -psi1, d = 1 - psi2;
  const double idet = 1.0 / (a * d - b * c);
  F.S00 = d * idet; F.S01 = -b * idet; F.S10 = -c * idet; F.S11 = a * idet;
}

// W⁻¹ applied to W.r in place
template <int NS, typename ST>
__device__ __forceinline__ void solve_W(WarpMem<NS, ST>& W, const Factor<NS, ST>& F, const double* cv, const double* w,
                                        const ModelDesc& M) {
  const int lane = threadIdx.x & 31;
  solve_M(W, M, F.is, F.ihc);
  double psi, rho;
  functionals(W.r, w, M, psi, rho);
  const double ph = phidot(cv, rho, (double)W.r[0], psi);
  const ST t0 = (ST)(F.S00 * ph + F.S01 * psi), t1 = (ST)(F.S10 * ph + F.S11 * psi);
  __syncwarp();
#pragma unroll
  for (int sl = 0; sl < NS; ++sl) {
    const int i = lane + 32 * sl;
    if (i < M.n) W.r[i] = W.r[i] + W.Z1[i] * t0 + W.Z2[i] * t1;
  }
  __syncwarp();
}

// U = W⁻¹ b with optional FP64 iterative refinement (W = s I - J at the step start).
template <int NS, typename ST>
__device__ void stage_solve(WarpMem<NS, ST>& W, const Factor<NS, ST>& F, const Coef& CJ, const CompDesc* __restrict__ comps,
                            const ModelDesc& M, double k, double s, int refine, const double (&b)[NS], double (&U)[NS]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int sl = 0; sl < NS; ++sl) { const int i = lane + 32 * sl; if (i < M.n) W.r[i] = (ST)b[sl]; }
  __syncwarp();
  solve_W(W, F, CJ.cv, CJ.w, M);
#pragma unroll
  for (int sl = 0; sl < NS; ++sl) { const int i = lane + 32 * sl; U[sl] = (i < M.n) ? (double)W.r[i] : 0.0; }
  for (int it = 0; it < refine; ++it) {
#pragma unroll
    for (int sl = 0; sl < NS; ++sl) { const int i = lane + 32 * sl; if (i < M.n) W.x[i] = U[sl]; }
    __syncwarp();
    double JU[NS];
    matvec(W, W.x, CJ.cv, CJ.w, comps, M, k, JU);
    __syncwarp();
#pragma unroll
    for (int sl = 0; sl < NS; ++sl) {
      const int i = lane + 32 * sl;
      if (i < M.n) W.r[i] = (ST)(b[sl] - (s * U[sl] - JU[sl]));
    }
    __syncwarp();
    solve_W(W, F, CJ.cv, CJ.w, M);
#pragma unroll
    for (int sl = 0; sl < NS; ++sl) { const int i = lane + 32 * sl; if (i < M.n) U[sl] += (double)W.r[i]; }
  }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  return v;
}

// ------------------------------------------------------------------------------------------
// outputs at one saved time τ for state y (in W.x)
template <int NS, typename ST>
__device__ void emit_output(WarpMem<NS, ST>& W, const PtArgs& A, const CosmoDesc* cd, const double* tab,
                            const CompDesc* __restrict__ comps, const ModelDesc& M, double k, double tau,
                            const double (&y)[NS], int item, int j) {
  const int lane = threadIdx.x & 31;
  if (A.output == SBZ_OUT_STATE) {
    double* o = A.out + ((size_t)item * A.ntau + j) * M.n;
#pragma unroll
    for (int sl = 0; sl < NS; ++sl) { const int i = lane + 32 * sl; if (i < M.n) o[i] = y[sl]; }
    return;
  }
  if (A.output != SBZ_OUT_SOURCES) return;
  // line-of-sight sources (src/models/cosmologies.jl:99-105)
  Coef CS{W.cvS, W.cvdS, W.wS, W.wdS};
  coef_eval(W, CS, cd, tab, M.nexpr, M.nx, k, tau, true, true);
#pragma unroll
  for (int sl = 0; sl < NS; ++sl) { const int i = lane + 32 * sl; if (i < M.n) W.x[i] = y[sl]; }
  __syncwarp();
  double fy[NS], dJy[NS], Jf[NS], phid, psi, dpsi_w;
  matvec(W, W.x, CS.cv, CS.w, comps, M, k, fy, &phid, &psi);
  matvec_dtau(W, W.x, CS, comps, M, k, dJy, &dpsi_w);
#pragma unroll
  for (int sl = 0; sl < NS; ++sl) { const int i = lane + 32 * sl; if (i < M.n) W.f[i] = fy[sl]; }
  __syncwarp();
  double psi_f, rho_f;
  functionals(W.f, CS.w, M, psi_f, rho_f);
  matvec(W, W.f, CS.cv, CS.w, comps, M, k, Jf);
  // second derivative of Π = F2 + G0 + G2 along the flow: (J'y + J f) restricted to those rows
  double g = 0;
  if (lane == 7 || lane == 8 || lane == 10) g = dJy[0] + Jf[0];
  const double Pidd = warp_sum(g);
  __syncwarp();
  if (lane == 0) {
    const double ek = W.src[0], kdd = W.src[1], kddd = W.src[2];
    const double kd = W.B[B_KD];
    const double v = -kd * ek, vd = (kd * kd - kdd) * ek, vdd = (-kd * kd * kd + 3 * kd * kdd - kddd) * ek;
    const double Pi = W.x[7] + W.x[8] + W.x[10];
    const double Pid = W.f[7] + W.f[8] + W.f[10];
    const double psid = dpsi_w + psi_f;  // Ψ' = (∂Ψ/∂τ) y + Ψ(f)
    const double sT = v * (W.x[5] * 0.25 + psi + Pi / 16) + ek * (psid + phid) + (vd * W.x[4] + v * W.f[4]) / (k * k) +
                      3.0 / (16.0 * k * k) * (vdd * Pi + 2 * vd * Pid + v * Pidd);
    const double chi = cd->tau0 - tau;
    const double SE = 3.0 / 16.0 * v * Pi / ((k * chi) * (k * chi));
    const double Spsi = (tau >= cd->taurec) ? -(psi + W.x[0]) * (tau - cd->taurec) / (cd->tau0 - cd->taurec) / chi : 0.0;
    double* o = A.out + ((size_t)item * A.ntau + j) * 3;
    o[0] = k * sT; o[1] = k * k * SE; o[2] = Spsi;
  }
  __syncwarp();
}

template <int NS, typename ST>
__global__ void __launch_bounds__(128) pt_kernel(PtArgs A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  ModelDesc& M = *reinterpret_cast<ModelDesc*>(smem_raw);
  CompDesc* comps = reinterpret_cast<CompDesc*>(smem_raw + ((sizeof(ModelDesc) + 15) & ~size_t(15)));
  const size_t comp_bytes = ((size_t)A.model_n * sizeof(CompDesc) + 15) & ~size_t(15);
  WarpMem<NS, ST>* Wm = reinterpret_cast<WarpMem<NS, ST>*>(smem_raw + ((sizeof(ModelDesc) + 15) & ~size_t(15)) + comp_bytes);
  WarpMem<NS, ST>& W = Wm[warp];
  // block-wide copy of the model descriptors
  for (int i = threadIdx.x; i < (int)sizeof(ModelDesc) / 4; i += blockDim.x) reinterpret_cast<int*>(&M)[i] = reinterpret_cast<const int*>(A.model)[i];
  for (int i = threadIdx.x; i < A.model_n * (int)sizeof(CompDesc) / 4; i += blockDim.x) reinterpret_cast<int*>(comps)[i] = reinterpret_cast<const int*>(A.comps)[i];
  __syncthreads();
  const int n = M.n;
  for (int i = lane; i < kNCV; i += 32) { W.cvJ[i] = W.cvdJ[i] = W.cvS[i] = W.cvdS[i] = 0; }
  for (int i = lane; i < kWF; i += 32) { W.wJ[i] = W.wdJ[i] = W.wS[i] = W.wdS[i] = 0; }
  for (int i = n + lane; i <= 32 * NS; i += 32) { W.x[i] = 0; W.f[i] = 0; W.r[i] = 0; }
  __syncwarp();
  Coef CJ{W.cvJ, W.cvdJ, W.wJ, W.wdJ}, CS{W.cvS, W.cvdS, W.wS, W.wdS};
  const double rtol = A.rtol, atol = A.atol;
  (void)nwarps;

  for (;;) {
    int slot = 0;
    if (lane == 0) slot = (int)atomicAdd(A.counter, 1u);
    slot = __shfl_sync(FULL, slot, 0);
    if (slot >= A.nitems) break;
    const int item = A.order ? A.order[slot] : slot;
    const int c = A.item_cosmo ? A.item_cosmo[item] : 0;
    const CosmoDesc* cd = A.cosmos + c;
    const double* tab = A.tables + (size_t)c * A.table_stride;
    const double* taus = A.taus ? A.taus + (size_t)c * A.ntau : nullptr;
    const double k = A.item_k[item];
    const double tend = cd->tau0;
    double t = fmin(fmax(A.item_tau_ini[item], cd->tau_start), tend);
    int status = SBZ_OK;
    int64_t nacc = 0, nrej = 0;
    double y[NS], f0[NS], ft[NS];

    // ---- adiabatic initial conditions (src/models/cosmologies.jl:74-77 and species ieqs) ----
    coef_eval(W, CS, cd, tab, M.nexpr, M.nx, k, t, false, false);
    {
      const double a = 1.0 / W.B[B_IA], kdv = W.B[B_KD];
      double Ir = 0;
      if (lane < M.nx) Ir = cd->Wq[lane] * W.B[B_E + lane];
      Ir = warp_sum(Ir);
      const double rg = cd->Og0, rn = cd->On0 + cd->wh * Ir;  // × a⁻⁴
      const double fnu = rn / (rg + rn);
      const double Psi = 10.0 / (15.0 + 4.0 * fnu);
      const double kt = k * t;
      const double F1 = 2.0 / 3.0 * kt * Psi;
      const double F2 = -8.0 / 15.0 * k / kdv * F1;
      const double G2 = F2 / 16.0;
      const double N2 = 2.0 / 15.0 * kt * kt * Psi;
      (void)a;
#pragma unroll
      for (int sl = 0; sl < NS; ++sl) {
        const int i = lane + 32 * sl;
        double v = 0;
        if (i < n) {
          if (i == 1 || i == 3) v = -1.5 * Psi;
          else if (i == 2 || i == 4) v = 0.5 * k * kt * Psi;
          else if (i == 5) v = -2 * Psi;
          else if (i == 6) v = F1;
          else if (i == 7) v = F2;
          else if (i == 8) v = 5.0 / 16.0 * F2;
          else if (i == 9) v = -1.0 / 16.0 * k / kdv * F2;
          else if (i == 10) v = G2;
          else if (i == M.oFt) v = -3.0 / 7.0 * k / kdv * F2;
          else if (i == M.oGt) v = -3.0 / 7.0 * k / kdv * G2;
          else if (i == M.oN) v = -2 * Psi;
          else if (i == M.oN + 1) v = 2.0 / 3.0 * kt * Psi;
          else if (i == M.oN + 2) v = N2;
          else if (i == M.oN + 3) v = 3.0 / 7.0 * kt * N2;
          else if (i >= M.oH) {
            const int j = (i - M.oH) / (M.Lh + 1), l = (i - M.oH) - j * (M.Lh + 1);
            const double dl = cd->dlnf[j];
            if (l == 0) v = 0.5 * Psi * dl;
            else if (l == 1) v = -1.0 / 3.0 * W.B[B_IQ + j] * (0.5 * kt * Psi) * dl;
            else if (l == 2) v = -0.5 * (1.0 / 15.0 * kt * kt * Psi) * dl;
          }
        }
        y[sl] = v;
        if (i < n) W.x[i] = v;
      }
      __syncwarp();
      // Φ from k²(Φ - Ψ) = 12πa²Π with the initial shears: Ψ(y) is linear with unit weight on Φ
      double psi0, rho0;
      functionals(W.x, CS.w, M, psi0, rho0);  // Φ slot still 0
      if (lane == 0) y[0] = Psi - psi0;
      __syncwarp();
      if (lane == 0) W.x[0] = y[0];
      __syncwarp();
    }
    // outputs at or before the initial time
    int jout = 0;
    if (taus) {
      while (jout < A.ntau && taus[jout] <= t) {
        if (taus[jout] < t) {  // before the mode starts: zero
          if (A.output == SBZ_OUT_SOURCES && lane < 3) A.out[((size_t)item * A.ntau + jout) * 3 + lane] = 0;
          if (A.output == SBZ_OUT_STATE) for (int i = lane; i < n; i += 32) A.out[((size_t)item * A.ntau + jout) * n + i] = 0;
        } else {
          emit_output(W, A, cd, tab, comps, M, k, t, y, item, jout);
        }
        ++jout;
      }
    }

    // ---- integration ----
    if (t < tend) {
      coef_eval(W, CJ, cd, tab, M.nexpr, M.nx, k, t, true, false);
#pragma unroll
      for (int sl = 0; sl < NS; ++sl) { const int i = lane + 32 * sl; if (i < n) W.x[i] = y[sl]; }
      __syncwarp();
      matvec(W, W.x, CJ.cv, CJ.w, comps, M, k, f0);
      // initial step (Hairer-Nørsett-Wanner II.4)
      double h;
      {
        double d0 = 0, d1 = 0;
#pragma unroll
        for (int sl = 0; sl < NS; ++sl) {
          const int i = lane + 32 * sl;
          if (i < n) { const double sk = atol + fabs(y[sl]) * rtol; d0 += (y[sl] / sk) * (y[sl] / sk); d1 += (f0[sl] / sk) * (f0[sl] / sk); }
        }
        d0 = sqrt(warp_sum(d0) / n); d1 = sqrt(warp_sum(d1) / n);
        double h0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * d0 / d1;
        h0 = fmin(h0, tend - t);
        __syncwarp();
#pragma unroll
        for (int sl = 0; sl < NS; ++sl) { const int i = lane + 32 * sl; if (i < n) W.x[i] = y[sl] + h0 * f0[sl]; }
        coef_eval(W, CS, cd, tab, M.nexpr, M.nx, k, t + h0, false, false);
        double f1[NS];
        matvec(W, W.x, CS.cv, CS.w, comps, M, k, f1);
        double d2 = 0;
#pragma unroll
        for (int sl = 0; sl < NS; ++sl) {
          const int i = lane + 32 * sl;
          if (i < n) { const double sk = atol + fabs(y[sl]) * rtol; const double q = (f1[sl] - f0[sl]) / (h0 * sk); d2 += q * q; }
        }
        d2 = sqrt(warp_sum(d2) / n);
        const double mx = fmax(d1, d2);
        const double h1 = (mx <= 1e-15 || !isfinite(mx)) ? fmax(1e-6, 1e-3 * h0) : pow(0.01 / mx, 0.2);
        h = fmin(100 * h0, h1);
        if (!isfinite(h) || h <= 0) h = 1e-6 * fmax(1.0, t);
      }
      double errold = 1e-4;
      bool rejected = false, nonfinite = false, have_jac = false;
      Factor<NS, ST> F;
      double hfac = 0;  // h used for the current factorisation
      int64_t iters = 0;
      while (t < tend) {
        if (++iters > A.maxiters) { status = SBZ_MAXITERS; break; }
        if (t + 1.01 * h >= tend) h = tend - t;
        if (!(h > 1e-14 * t)) { status = nonfinite ? SBZ_NONFINITE : SBZ_DTMIN; break; }
        if (!have_jac) {
          // J, ∂f/∂τ at the step start
#pragma unroll
          for (int sl = 0; sl < NS; ++sl) { const int i = lane + 32 * sl; if (i < n) W.x[i] = y[sl]; }
          __syncwarp();
          matvec_dtau(W, W.x, CJ, comps, M, k, ft);
          have_jac = true;
          hfac = 0;
        }
        const double s = 1.0 / (h * rw::gam), ih = 1.0 / h;
        if (h != hfac) { factorize(W, F, CJ.cv, CJ.w, comps, M, k, s); hfac = h; }
        double U1[NS], U2[NS], U3[NS], U4[NS], U5[NS], U6[NS], b[NS], Fv[NS];
#pragma unroll
        for (int sl = 0; sl < NS; ++sl) b[sl] = f0[sl] + h * rw::d1 * ft[sl];
        stage_solve(W, F, CJ, comps, M, k, s, A.refine, b, U1);
        // stage 2
#pragma unroll
        for (int sl = 0; sl < NS; ++sl) { const int i = lane + 32 * sl; if (i < n) W.x[i] = y[sl] + rw::A21 * U1[sl]; }
        coef_eval(W, CS, cd, tab, M.nexpr, M.nx, k, t + rw::c2 * h, false, false);
        matvec(W, W.x, CS.cv, CS.w, comps, M, k, Fv);
#pragma unroll
        for (int sl = 0; sl < NS; ++sl) b[sl] = Fv[sl] + ih * (rw::C21 * U1[sl]) + h * rw::d2 * ft[sl];
        stage_solve(W, F, CJ, comps, M, k, s, A.refine, b, U2);
        // stage 3
#pragma unroll
        for (int sl = 0; sl < NS; ++sl) { const int i = lane + 32 * sl; if (i < n) W.x[i] = y[sl] + rw::A31 * U1[sl] + rw::A32 * U2[sl]; }
        coef_eval(W, CS, cd, tab, M.nexpr, M.nx, k, t + rw::c3 * h, false, false);
        matvec(W, W.x, CS.cv, CS.w, comps, M, k, Fv);
#pragma unroll
        for (int sl = 0; sl < NS; ++sl) b[sl] = Fv[sl] + ih * (rw::C31 * U1[sl] + rw::C32 * U2[sl]) + h * rw::d3 * ft[sl];
        stage_solve(W, F, CJ, comps, M, k, s, A.refine, b, U3);
        // stage 4
#pragma unroll
        for (int sl = 0; sl < NS; ++sl) { const int i = lane + 32 * sl; if (i < n) W.x[i] = y[sl] + rw::A41 * U1[sl] + rw::A42 * U2[sl] + rw::A43 * U3[sl]; }
        coef_eval(W, CS, cd, tab, M.nexpr, M.nx, k, t + rw::c4 * h, false, false);
        matvec(W, W.x, CS.cv, CS.w, comps, M, k, Fv);
#pragma unroll
        for (int sl = 0; sl < NS; ++sl) b[sl] = Fv[sl] + ih * (rw::C41 * U1[sl] + rw::C42 * U2[sl] + rw::C43 * U3[sl]) + h * rw::d4 * ft[sl];
        stage_solve(W, F, CJ, comps, M, k, s, A.refine, b, U4);
        // stage 5 (at t + h)
        const double tn = (h == tend - t) ? tend : t + h;
        double Y[NS];
#pragma unroll
        for (int sl = 0; sl < NS; ++sl) {
          const int i = lane + 32 * sl;
          Y[sl] = y[sl] + rw::A51 * U1[sl] + rw::A52 * U2[sl] + rw::A53 * U3[sl] + rw::A54 * U4[sl];
          if (i < n) W.x[i] = Y[sl];
        }
        coef_eval(W, CS, cd, tab, M.nexpr, M.nx, k, tn, true, false);
        matvec(W, W.x, CS.cv, CS.w, comps, M, k, Fv);
#pragma unroll
        for (int sl = 0; sl < NS; ++sl) b[sl] = Fv[sl] + ih * (rw::C51 * U1[sl] + rw::C52 * U2[sl] + rw::C53 * U3[sl] + rw::C54 * U4[sl]);
        stage_solve(W, F, CJ, comps, M, k, s, A.refine, b, U5);
        // stage 6
        __syncwarp();
#pragma unroll
        for (int sl = 0; sl < NS; ++sl) { const int i = lane + 32 * sl; Y[sl] += U5[sl]; if (i < n) W.x[i] = Y[sl]; }
        __syncwarp();
        matvec(W, W.x, CS.cv, CS.w, comps, M, k, Fv);
#pragma unroll
        for (int sl = 0; sl < NS; ++sl) b[sl] = Fv[sl] + ih * (rw::C61 * U1[sl] + rw::C62 * U2[sl] + rw::C63 * U3[sl] + rw::C64 * U4[sl] + rw::C65 * U5[sl]);
        stage_solve(W, F, CJ, comps, M, k, s, A.refine, b, U6);
        // error estimate and new state
        double e2 = 0, y1[NS];
#pragma unroll
        for (int sl = 0; sl < NS; ++sl) {
          const int i = lane + 32 * sl;
          y1[sl] = Y[sl] + U6[sl];
          if (i < n) { const double sk = atol + rtol * fmax(fabs(y[sl]), fabs(y1[sl])); const double q = U6[sl] / sk; e2 += q * q; }
        }
        const double err = sqrt(warp_sum(e2) / n);
        if (isfinite(err) && err <= 1.0) {
          // accept: f(t1, y1) with the t1 coefficients (CS holds them), then dense output
          __syncwarp();
#pragma unroll
          for (int sl = 0; sl < NS; ++sl) { const int i = lane + 32 * sl; if (i < n) W.x[i] = y1[sl]; }
          __syncwarp();
          double f1[NS];
          matvec(W, W.x, CS.cv, CS.w, comps, M, k, f1);
          // the t1 coefficient set becomes the next step's Jacobian set
#pragma unroll
          for (int q = lane; q < kNCV; q += 32) { W.cvJ[q] = W.cvS[q]; W.cvdJ[q] = W.cvdS[q]; }
          for (int q = lane; q < kWF; q += 32) { W.wJ[q] = W.wS[q]; W.wdJ[q] = W.wdS[q]; }
          __syncwarp();
          if (taus) {
            while (jout < A.ntau && taus[jout] <= tn) {
              const double tau = taus[jout];
              const double hh = tn - t, sx = (tau - t) / hh, s2 = sx * sx, s3 = s2 * sx;
              const double h00 = 2 * s3 - 3 * s2 + 1, h10 = s3 - 2 * s2 + sx, h01 = 3 * s2 - 2 * s3, h11 = s3 - s2;
              double yo[NS];
#pragma unroll
              for (int sl = 0; sl < NS; ++sl) yo[sl] = h00 * y[sl] + h10 * hh * f0[sl] + h01 * y1[sl] + h11 * hh * f1[sl];
              emit_output(W, A, cd, tab, comps, M, k, tau, yo, item, jout);
              ++jout;
            }
          }
          t = tn;
#pragma unroll
          for (int sl = 0; sl < NS; ++sl) { y[sl] = y1[sl]; f0[sl] = f1[sl]; }
          ++nacc;
          double fac = 0.9 * pow(fmax(err, 1e-10), -0.175) * pow(errold, 0.1);
          fac = fmin(10.0, fmax(0.2, fac));
          if (rejected) fac = fmin(fac, 1.0);
          errold = fmax(err, 1e-4);
          h *= fac;
          rejected = false; nonfinite = false; have_jac = false;
        } else {
          ++nrej;
          rejected = true;
          if (!isfinite(err)) { nonfinite = true; h *= 0.2; }
          else h *= fmax(0.2, 0.9 * pow(err, -0.25));
          // CJ (coefficients at t) and ∂f/∂τ stay valid; only the factorisation changes
        }
      }
    }
    // saved times never reached (failed mode): zero
    if (taus) {
      for (; jout < A.ntau; ++jout) {
        if (A.output == SBZ_OUT_SOURCES && lane < 3) A.out[((size_t)item * A.ntau + jout) * 3 + lane] = 0;
        if (A.output == SBZ_OUT_STATE) for (int i = lane; i < n; i += 32) A.out[((size_t)item * A.ntau + jout) * n + i] = 0;
      }
    }
    bool finite = true;
#pragma unroll
    for (int sl = 0; sl < NS; ++sl) { const int i = lane + 32 * sl; if (i < n && !isfinite(y[sl])) finite = false; }
    finite = __all_sync(FULL, finite);
    if (status == SBZ_OK && !finite) status = SBZ_NONFINITE;
    if (A.output == SBZ_OUT_DELTA_M) {
      // Δ_m(τ0) = Σ ρ_s Δ_s / Σ ρ_s over c, b, massive ν   (src/observables/fourier.jl:39-52)
      coef_eval(W, CS, cd, tab, M.nexpr, M.nx, k, tend, false, false);
#pragma unroll
      for (int sl = 0; sl < NS; ++sl) { const int i = lane + 32 * sl; if (i < n) W.x[i] = y[sl]; }
      __syncwarp();
      double I0 = 0, I1 = 0, Ir = 0;
      if (lane < M.nx) {
        const int base = M.oH + lane * (M.Lh + 1);
        I0 = cd->Wq[lane] * W.B[B_E + lane] * W.x[base];
        I1 = cd->Wq[lane] * cd->xq[lane] * W.x[base + 1];
        Ir = cd->Wq[lane] * W.B[B_E + lane];
      }
      I0 = warp_sum(I0); I1 = warp_sum(I1); Ir = warp_sum(Ir);
      if (lane == 0) {
        const double ia = W.B[B_IA], Hc = W.B[B_H];
        const double ik2 = 1.0 / (k * k);
        double num = cd->Oc0 * (W.x[1] + 3 * Hc * W.x[2] * ik2) + cd->Ob0 * (W.x[3] + 3 * Hc * W.x[4] * ik2);
        double den = cd->Oc0 + cd->Ob0;
        num += cd->wh * ia * (I0 + 3 * Hc * I1 / k);
        den += cd->wh * ia * Ir;
        A.out[item] = num / den;
      }
      __syncwarp();
    }
    if (lane == 0) {
      if (A.status) A.status[item] = status;
      if (A.steps) { A.steps[2 * item] = nacc; A.steps[2 * item + 1] = nrej; }
    }
    __syncwarp();
  }
}

template <int NS, typename ST>
int launch_ns(const PtArgs& A, int warps_per_block, int num_sms, cudaStream_t stream) {
  const size_t head = ((sizeof(ModelDesc) + 15) & ~size_t(15)) + (((size_t)A.model_n * sizeof(CompDesc) + 15) & ~size_t(15));
  const size_t smem = head + warps_per_block * sizeof(WarpMem<NS, ST>);
  auto kern = pt_kernel<NS, ST>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return SBZ_ERR_CUDA;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * warps_per_block, smem) != cudaSuccess) return SBZ_ERR_CUDA;
  per_sm = per_sm < 1 ? 1 : per_sm;
  const int want = (A.nitems + warps_per_block - 1) / warps_per_block;
  const int grid = want < num_sms * per_sm ? want : num_sms * per_sm;
  kern<<<grid > 0 ? grid : 1, 32 * warps_per_block, smem, stream>>>(A);
  return cudaGetLastError() == cudaSuccess ? SBZ_OK : SBZ_ERR_CUDA;
}


// f = J(τ) y and ∂f/∂τ = (dJ/dτ) y for single modes (one warp each): the model's right-hand side
// as the integrator evaluates it.
template <int NS, typename ST>
__global__ void __launch_bounds__(32) rhs_kernel(PtArgs A, const double* __restrict__ y_in, const double* __restrict__ tau_in,
                                                 double* __restrict__ f_out, double* __restrict__ ft_out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  ModelDesc& M = *reinterpret_cast<ModelDesc*>(smem_raw);
  CompDesc* comps = reinterpret_cast<CompDesc*>(smem_raw + ((sizeof(ModelDesc) + 15) & ~size_t(15)));
  const size_t comp_bytes = ((size_t)A.model_n * sizeof(CompDesc) + 15) & ~size_t(15);
  WarpMem<NS, ST>& W = *reinterpret_cast<WarpMem<NS, ST>*>(smem_raw + ((sizeof(ModelDesc) + 15) & ~size_t(15)) + comp_bytes);
  for (int i = lane; i < (int)sizeof(ModelDesc) / 4; i += 32) reinterpret_cast<int*>(&M)[i] = reinterpret_cast<const int*>(A.model)[i];
  for (int i = lane; i < A.model_n * (int)sizeof(CompDesc) / 4; i += 32) reinterpret_cast<int*>(comps)[i] = reinterpret_cast<const int*>(A.comps)[i];
  __syncwarp();
  const int n = M.n, item = blockIdx.x;
  for (int i = lane; i < kNCV; i += 32) { W.cvS[i] = W.cvdS[i] = 0; }
  for (int i = lane; i < kWF; i += 32) { W.wS[i] = W.wdS[i] = 0; }
  for (int i = n + lane; i <= 32 * NS; i += 32) W.x[i] = 0;
  __syncwarp();
  const int c = A.item_cosmo ? A.item_cosmo[item] : 0;
  const CosmoDesc* cd = A.cosmos + c;
  const double* tab = A.tables + (size_t)c * A.table_stride;
  const double k = A.item_k[item], tau = tau_in[item];
  Coef CS{W.cvS, W.cvdS, W.wS, W.wdS};
  coef_eval(W, CS, cd, tab, M.nexpr, M.nx, k, tau, true, false);
  for (int i = lane; i < n; i += 32) W.x[i] = y_in[(size_t)item * n + i];
  __syncwarp();
  double f[NS], ft[NS];
  matvec(W, W.x, CS.cv, CS.w, comps, M, k, f);
  matvec_dtau(W, W.x, CS, comps, M, k, ft);
#pragma unroll
  for (int sl = 0; sl < NS; ++sl) {
    const int i = lane + 32 * sl;
    if (i < n) { f_out[(size_t)item * n + i] = f[sl]; ft_out[(size_t)item * n + i] = ft[sl]; }
  }
}

template <int NS>
int rhs_launch_ns(const PtArgs& A, const double* y, const double* tau, double* f, double* ft, cudaStream_t st) {
  const size_t smem = ((sizeof(ModelDesc) + 15) & ~size_t(15)) + (((size_t)A.model_n * sizeof(CompDesc) + 15) & ~size_t(15)) +
                      sizeof(WarpMem<NS, double>);
  auto kern = rhs_kernel<NS, double>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return SBZ_ERR_CUDA;
  kern<<<A.nitems, 32, smem, st>>>(A, y, tau, f, ft);
  return cudaGetLastError() == cudaSuccess ? SBZ_OK : SBZ_ERR_CUDA;
}

}  // namespace ptk
}  // namespace sbz
