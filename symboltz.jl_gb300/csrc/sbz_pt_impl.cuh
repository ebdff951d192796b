#pragma once
// Perturbation solver kernel (implementation; instantiated in sbz_pt_f32*.cu / sbz_pt_f64*.cu):
// a group of NW warps integrates one (cosmology, k) mode.
//
// Replaces the per-k loop of solvept (src/solve.jl:543-569) and the Rodas5P + KLU inner solver
// it calls (src/solve.jl:327-341).  Integrator: Rodas5P (Rosenbrock, order 5(4), stiffly
// accurate; tableau in sbz_rosenbrock.cuh) in transformed form
//   (1/(hγ) - J) U_i = f(t+c_i h, y + Σ A_ij U_j) + Σ (C_ij/h) U_j + h d_i ∂f/∂τ,
//   y1 = y + Σ_{j<8} A_8j U_j + U_8, error estimate U_8,
// with the error norm, PI step-size control and an order-4 continuous extension for the saved
// times.  The perturbation system is linear, u' = J(τ) u, so "f" and "J·x" are one operator; its
// rows are described in sbz_layout.hpp.
//
// Stage solves exploit the structure of M = 1/(hγ) - B (J = B + c_Φ̇ ∇Φ̇ᵀ + c_Ψ ∇Ψᵀ):
//   * the free-streaming hierarchies are tridiagonal chains, eliminated from their truncation end
//     by warp scans (no pivoting needed: pivots stay ≥ 1/(hγ));
//   * photon-baryon rows δb, θb, F0-2, G0-2 form a dense 8x8 head (explicit inverse, partial pivoting);
//   * CDM and Φ are 2x2/1x1 triangular blocks;
//   * the two metric couplings are added back with a rank-2 Sherman-Morrison-Woodbury update.
// ST = double: all-FP64 solve.  ST = float: FP32 factorisation and solves with FP64 iterative
// refinement against the FP64 operator (residuals, state, error norm and step control in FP64).
//
// Work split: the mode's components i = gt + NT·s (NT = 32·NW threads, s < NSL slots) live in
// registers of thread gt.  On GB300 an FP64 warp instruction holds an SM sub-partition's FP64
// pipe for ~64 cycles, so a single mode's step latency is set by the FP64 instruction count per
// warp; NW = 4 spreads one mode over the four sub-partitions of an SM, which is what bounds the
// slowest (high-k) modes of a spectrum.  The group synchronises with a named barrier (NW > 1) or
// __syncwarp (NW = 1); every barrier sits in group-uniform control flow.  Step control (the PI
// controller, 1/h, 1/(hγ), the stage times) runs on one warp and reaches the others through shared
// memory at the loop-top barrier.  Wide groups run the stage loop rolled with the stage vectors in
// shared memory (kRolledStages), narrow ones unrolled with them in registers.  Loops are bounded by
// opts.maxiters and a step-size floor, so a mode that cannot finish sets a status code and the
// group moves on.
#include <cuda_runtime.h>
#include <cstdint>
#include "sbz_layout.hpp"
#include "sbz_pt.cuh"
#include "sbz_rosenbrock.cuh"

namespace sbz {
namespace ptk {

constexpr unsigned FULL = 0xffffffffu;

using TB = ros::Rodas5P;  // the integrator's tableau

constexpr int kWF = 2 * kMaxFun;  // functional weights per set: Ψ terms then δρ terms
constexpr int kMaxT = TB::NTIME;  // coefficient sets evaluated in one call (the later stage times)
constexpr int kNSets = TB::NTIME + 2;  // J (step start), the later stage times (the last is the step end), output time

static_assert(sizeof(ModelDesc) % 4 == 0 && sizeof(CompDesc) % 4 == 0 && sizeof(CosmoDesc) % 4 == 0, "word copies");

// The tableau as a constant-memory table for the rolled stage loop of wide groups (stage index
// uniform over the group: broadcast reads).
struct RosTab {
  double A[TB::S][TB::S], C[TB::S][TB::S], d[TB::S];
  int tslot[TB::S], hasd[TB::S], incr[TB::S];
  int nst;
  constexpr RosTab() : A{}, C{}, d{}, tslot{}, hasd{}, incr{}, nst(TB::S) {
    for (int i = 0; i < TB::S; ++i) {
      for (int j = 0; j < TB::S; ++j) { A[i][j] = TB::A(i, j); C[i][j] = TB::C(i, j); }
      d[i] = TB::d(i); tslot[i] = TB::tslot(i); hasd[i] = TB::d(i) != 0.0; incr[i] = TB::incremental(i);
    }
  }
};
static __constant__ RosTab kRos = RosTab();
// Groups of four or more warps, and two-warp groups in mixed precision, run the stage loop rolled,
// one copy of the stage body, so the step's code stays in the instruction cache (the unrolled loop
// streamed it: the 1000-mode spectrum went from 1,788 to 1,721 ms with four-warp groups, the
// batched 256-cosmology solve from 80.7 to 65.1 s with two-warp groups); the stage solutions then
// live in shared memory.  Narrower groups keep the unrolled loop with the stages in registers:
// there shared memory sets the occupancy (the all-FP64 two-warp batch ran 119 s unrolled against
// 150 s for the best rolled shape).
template <int NW, typename ST>
constexpr bool kRolledStages = NW >= 4 || (NW >= 2 && sizeof(ST) == 4);

// one coefficient set: operator coefficients, their τ-derivatives, functional weights
struct CSet {
  double cv[kNCV], cvd[kNCV], w[kWF], wd[kWF];
};

template <int NW, int NSL, typename ST>
struct ModeMem {
  static constexpr int NT = 32 * NW, NM = NT * NSL;
  double x[NM + 1];   // operator input; x[n..NM] stay 0
  double f[NM + 1];
  ST r[NM + 1];       // structured-solve right-hand side / work vector
  ST dinv[NM], sub[NM], sup[NM], mfw[NM], dd[NM];
  ST fA[5][NM], bA[5][NM], bP[NM];   // warp-scan multipliers of the chain eliminations, per row
  ST cf[2][kMaxChains];              // forward-eliminated first row of each chain, per vector
  int16_t att[NM];                   // head row a chain row's back substitution depends on, or -1
  int hatt[8];                       // chain attached to head row 3 + q, or -1
  int hfused;                        // every chain attached to the head is in pair 0 (warp 0's)
  ST Z1[NM + 1], Z2[NM + 1];
  ST H[64], Hinv[64];
  ST hmul[kMaxChains], hcorr[kMaxChains];
  ST wS[kWF], fS[4];  // Jacobian-set functional weights and Φ̇ coefficients in solve precision
  CSet cs[kNSets];
  double Us[kRolledStages<NW, ST> ? TB::S : 1][kRolledStages<NW, ST> ? NM : 1];  // stage solutions (rolled stage loop)
  double B[kMaxT][B_COUNT], dB[kMaxT][B_COUNT];
  double src[4];      // e^{-κ}, κ̈, κ⃛ at an output time
  double red[2][NW];  // ping-pong group reductions
  float redf[2][NW];
  double ctl[4 + kMaxT];  // step control from the controller warp: h, 1/h, 1/(hγ), step end, stage times
  int ctlf;               // and its flags
  CosmoDesc cdesc;    // the current mode's cosmology (coefficient expressions, bin momenta)
  int item;
};

// group of NW warps working on one mode
template <int NW>
struct Grp {
  int gt, lane, wq, bar;
  int fc;          // component of this lane's metric-functional term (n: none; x[n] == 0)
  unsigned pp;     // bit s: some row of slot s in this warp carries a Φ̇ or Ψ coupling
  mutable int rp;  // ping-pong reduction buffer
  __device__ __forceinline__ void sync() const {
    if constexpr (NW == 1) __syncwarp();
    else asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(NW * 32) : "memory");
  }
};

// Component held by thread gt in slot s.  Slot 0 is the identity (the head rows with their extra
// couplings sit in warp 0); slot s ≥ 1 is rotated by s·(NW-1) warps, so a partial last slot lands
// on warp 1 — for NW = 4 the warp of the photon tails, which carries no metric-coupled row and so
// skips the Ψ/Φ̇ functionals of every operator product — not on the head warp.
template <int NW>
__device__ __forceinline__ int comp_of(int gt, int s) { return s * 32 * NW + ((gt + 32 * (NW - 1) * s) & (32 * NW - 1)); }

// per-lane model constants kept in registers: the lane's functional component and, per slot,
// whether any row of this warp carries a Φ̇ or Ψ coupling (warp-uniform; the operator products skip
// those terms otherwise)
template <int NW, int NSL>
__device__ __forceinline__ void init_lane_consts(Grp<NW>& g, const ModelDesc& M, const CompDesc* comps) {
  const int l = g.lane;
  g.fc = l < M.npsi ? M.psiComp[l] : (l >= kMaxFun && l - kMaxFun < M.nrho) ? M.rhoComp[l - kMaxFun] : M.n;
  g.pp = 0;
#pragma unroll
  for (int s = 0; s < NSL; ++s) {
    const int i = comp_of<NW>(g.gt, s);
    const bool need = i < M.n && (comps[i].phid != CV_ZERO || comps[i].psid != CV_ZERO);
    if (__any_sync(FULL, need)) g.pp |= 1u << s;
  }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  return v;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  return v;
}

template <int NW, int NSL, typename ST, typename T>
__device__ __forceinline__ T group_sum(const Grp<NW>& g, ModeMem<NW, NSL, ST>& W, T v) {
  v = warp_sum(v);
  if constexpr (NW == 1) {
    __syncwarp();
    return v;
  } else {
    if (g.lane == 0) W.red[g.rp][g.wq] = v;
    g.sync();
    T s = 0;
#pragma unroll
    for (int w = 0; w < NW; ++w) s += (T)W.red[g.rp][w];
    g.rp ^= 1;
    return s;
  }
}

template <int NW, int NSL, typename ST>
__device__ __forceinline__ float group_max(const Grp<NW>& g, ModeMem<NW, NSL, ST>& W, float v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v = fmaxf(v, __shfl_xor_sync(FULL, v, o));
  if constexpr (NW == 1) {
    __syncwarp();
    return v;
  } else {
    if (g.lane == 0) W.redf[g.rp][g.wq] = v;
    g.sync();
    float s = 0;
#pragma unroll
    for (int w = 0; w < NW; ++w) s = fmaxf(s, W.redf[g.rp][w]);
    g.rp ^= 1;
    return s;
  }
}

// FP32 <-> FP64 conversions with integer operations.  The FP64 pipe of this GPU issues one warp
// instruction per 64 cycles, conversions and comparisons included, while these are a handful of
// integer-pipe instructions.  Both are exact for normal numbers and zero (FP64 -> FP32 rounds to
// nearest even, as the hardware conversion does); FP32 subnormals are flushed to zero, results
// beyond the FP32 range become ±inf, NaN stays NaN.
__device__ __forceinline__ double f32_to_f64(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu, sg = u & 0x80000000u;
  const unsigned de = e == 0xffu ? 0x7ffu : e + 896u;
  const unsigned hi = e == 0 ? sg : (sg | (de << 20) | ((u & 0x7fffffu) >> 3));
  const unsigned lo = e == 0 ? 0u : (u << 29);
  return __hiloint2double((int)hi, (int)lo);
}
__device__ __forceinline__ float f64_to_f32(double d) {
  const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
  const unsigned sg = hi & 0x80000000u, ex = (hi >> 20) & 0x7ffu;
  const int e = (int)ex - 896;
  const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29), rest = lo & 0x1fffffffu;
  unsigned r = ((unsigned)e << 23) + m;
  r += (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) ? 1u : 0u;  // a carry moves into the exponent
  r = e <= 0 ? 0u : (e >= 255 ? 0x7f800000u : r);
  if (ex == 0x7ffu) r = ((hi & 0xfffffu) | lo) ? 0x7fc00000u : 0x7f800000u;
  return __uint_as_float(sg | r);
}
template <typename ST>
__device__ __forceinline__ ST to_st(double v);
template <>
__device__ __forceinline__ float to_st<float>(double v) { return f64_to_f32(v); }
template <>
__device__ __forceinline__ double to_st<double>(double v) { return v; }
__device__ __forceinline__ double from_st(float v) { return f32_to_f64(v); }
__device__ __forceinline__ double from_st(double v) { return v; }
// Order of non-negative doubles (and NaN above +inf) by their bit patterns: integer comparisons.
__device__ __forceinline__ long long dkey(double v) { return __double_as_longlong(v); }
// Max / min of doubles of either sign through an order-preserving integer key (no NaN operands).
__device__ __forceinline__ long long okey(double v) {
  const long long b = __double_as_longlong(v);
  return b ^ ((b >> 63) & 0x7fffffffffffffffll);
}
__device__ __forceinline__ double dmax(double a, double b) { return okey(a) >= okey(b) ? a : b; }
__device__ __forceinline__ double dmin(double a, double b) { return okey(a) <= okey(b) ? a : b; }

template <typename ST>
__device__ __forceinline__ ST rcp(ST v);
template <>
__device__ __forceinline__ float rcp<float>(float v) {  // approximate reciprocal: the FP32 solve is a preconditioner
  float r;
  asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(v));
  return r;
}
template <>
__device__ __forceinline__ double rcp<double>(double v) { return 1.0 / v; }

struct ModeK {  // per-mode constants
  double k, k2, ik, ik2;
};

// ------------------------------------------------------------------------------------------
// Cubic Hermite interpolation of table quantity c at τ (value, and τ-derivative if want_d) from the
// interval's power-form coefficients (Horner: three FMAs for the value).  The node index comes from
// an FP32 logarithm and can be one off next to a node: every load of the guessed interval is issued
// at once and repeated only in that rare case.
__device__ __forceinline__ void table_cubic(const CosmoDesc* __restrict__ cd, const double* __restrict__ tab, double tau, int c,
                                            bool want_d, double& val, double& der) {
  const int ntab = cd->ntab;
  int gi = (int)((__logf(f64_to_f32(tau)) - cd->lnt0f) * cd->idlntf);
  gi = max(0, min(gi, ntab - 2));
  const double* nd = tab + (size_t)gi * kNodeStride;
  double t0 = nd[0], t1 = nd[kNodeStride], ih = nd[1];
  double a0 = nd[kNodePow + 4 * c], a1 = nd[kNodePow + 4 * c + 1], a2 = nd[kNodePow + 4 * c + 2], a3 = nd[kNodePow + 4 * c + 3];
  const long long kt = dkey(tau);  // τ and the node times are positive
  const int shift = (kt < dkey(t0) && gi > 0) ? -1 : (kt > dkey(t1) && gi < ntab - 2) ? 1 : 0;
  if (shift) {
    nd += shift * kNodeStride;
    t0 = nd[0]; ih = nd[1];
    a0 = nd[kNodePow + 4 * c]; a1 = nd[kNodePow + 4 * c + 1]; a2 = nd[kNodePow + 4 * c + 2]; a3 = nd[kNodePow + 4 * c + 3];
  }
  const double s = (tau - t0) * ih;
  val = fma(s, fma(s, fma(s, a3, a2), a1), a0);
  der = want_d ? fma(s, fma(s, 3.0 * a3, 2.0 * a2), a1) * ih : 0.0;
}

// ------------------------------------------------------------------------------------------
// τ-dependent coefficients at nt ≤ kMaxT times into sets cs[set[q]]; derivative sets where bit q
// of dmask is set.  source = true (nt = 1): also fetch e^{-κ}, κ̈, κ⃛ and use the Taylor-mode κ̈
// as dκ̇/dτ (the line-of-sight sources differentiate the background along its ODE,
// src/models/cosmologies.jl:99-105).  Warp p forms the base scalars of times 2p, 2p+1, lane =
// 16 (q - 2p) + c: lane c < 7 interpolates table quantity c at time q once; then every lane of the
// time takes one reciprocal square root, so the FP64 work is one instruction stream for all of
// them: lane 8 + j the energy of momentum bin j, E_j = sqrt(x_j² + (y0 a)²), lanes 5, 6, 7 the
// reciprocals 1/a, 1/ℋ, 1/τ as rsqrt(v²) (v > 0), with dr/dτ = -u r³, u = (1/2) dw/dτ for the
// derivative sets.  The expressions are then spread over the group.  The caller guarantees that no
// thread still reads the target sets; the call ends with a group barrier.
template <int NW, int NSL, typename ST>
__device__ __forceinline__ void coef_eval(const Grp<NW>& g, ModeMem<NW, NSL, ST>& W, const int* set, const double* taus, int nt,
                          unsigned dmask, bool source, const CosmoDesc* cd, const double* __restrict__ tab,
                          int nexpr, int nx, const ModeK& mk) {
  // times 2p, 2p+1 in pass p: warp p of the group, or every pass on the one warp when NW = 1
  for (int pass = NW == 1 ? 0 : g.wq; 2 * pass < nt; pass += NW) {
    const int lane = g.lane, q = 2 * pass + (lane >> 4), c = lane & 15;
    const bool live = q < nt;
    const bool dq = live && ((dmask >> q) & 1u);
    double v = 0, d = 0;
    if (live && c < 7) table_cubic(cd, tab, taus[q], c, dq, v, d);
    const int base = lane & ~15;
    const double a = __shfl_sync(FULL, v, base), da = __shfl_sync(FULL, d, base);
    const double hc = __shfl_sync(FULL, v, base + 1), dhc = __shfl_sync(FULL, d, base + 1);
    const double tq = live ? taus[q] : 1.0;
    double* Bq = W.B[live ? q : 0]; double* dBq = W.dB[live ? q : 0];
    const int j = c - 8;
    const bool bin = j >= 0 && j < nx;
    const double xj = bin ? cd->xq[j] : 0.0, ixj = bin ? cd->ixq[j] : 0.0;
    const double x = bin ? xj : c == 5 ? a : c == 6 ? hc : c == 7 ? tq : 1.0;
    const double dx = bin ? 0.0 : c == 5 ? da : c == 6 ? dhc : 1.0;
    const double ys = bin ? cd->y0 : 0.0;
    const double ya = ys * a;
    const double w = fma(x, x, ya * ya);
    const double r = rsqrt(w);
    const double E = w * r;
    const double p2 = (bin ? xj : r) * r;                     // bins: x_j / E; lane 5: 1/a²
    const double p3 = (bin ? E : cd->R0) * (bin ? ixj : r);  // bins: E / x_j; lane 5: R0 / a
    double ur = 0, dr = 0, dp2 = 0, dp3 = 0;
    if (dq) {
      const double u = fma(x, dx, ya * (ys * da));
      ur = u * r;                                   // bins: dE/dτ
      dr = -ur * (r * r);
      dp2 = (bin ? xj : r) * dr;                    // bins: d(x_j/E)/dτ; lane 5: half of d(1/a²)/dτ
      dp3 = (bin ? ur : cd->R0) * (bin ? ixj : dr);
    }
    if (live) {
      if (bin) {
        Bq[B_Q + j] = p2; Bq[B_IQ + j] = p3; Bq[B_E + j] = E; Bq[B_IE + j] = r;
        if (dq) { dBq[B_Q + j] = dp2; dBq[B_IQ + j] = dp3; dBq[B_E + j] = ur; dBq[B_IE + j] = dr; }
      } else if (c == 5) {
        Bq[B_IA] = r; Bq[B_IA2] = p2; Bq[B_R] = p3;
        if (dq) { dBq[B_IA] = dr; dBq[B_IA2] = 2.0 * dp2; dBq[B_R] = dp3; }
      } else if (c == 6) {
        Bq[B_IH] = r;
        if (dq) dBq[B_IH] = dr;
      } else if (c == 7) {
        Bq[B_ITAU] = r; Bq[B_ONE] = 1; Bq[B_K] = mk.k; Bq[B_K2] = mk.k2; Bq[B_IK] = mk.ik; Bq[B_IK2] = mk.ik2;
        if (dq) { dBq[B_ITAU] = dr; dBq[B_ONE] = 0; dBq[B_K] = 0; dBq[B_K2] = 0; dBq[B_IK] = 0; dBq[B_IK2] = 0; }
      }
      if (c == 1) {  // ℋ
        Bq[B_H] = v;
        if (dq) dBq[B_H] = d;
      } else if (c == 2) {  // κ̇ (for the sources, dκ̇/dτ is κ̈ from lane c = 5)
        Bq[B_KD] = v;
        if (dq && !source) dBq[B_KD] = d;
      } else if (c == 3) {  // c_s²
        Bq[B_CS2] = v;
        if (dq) dBq[B_CS2] = d;
      } else if (c >= 4 && c < 7 && source) {  // e^{-κ}, κ̈, κ⃛
        W.src[c - 4] = v;
        if (c == 5) dBq[B_KD] = v;
      }
    }
  }
  g.sync();
  // expression e at time q (with its τ-derivative when deriv): K1 p0 p1 p2 + K2 q0 q1 q2
  auto expr = [&](int q, int e, bool deriv) {
    const CoefExpr& X = cd->expr[e];
    const double* Bq = W.B[q];
    const double p0 = Bq[X.b[0]], p1 = Bq[X.b[1]], p2 = Bq[X.b[2]];
    const double q0 = Bq[X.b[3]], q1 = Bq[X.b[4]], q2 = Bq[X.b[5]];
    const double p12 = p1 * p2, q12 = q1 * q2;
    const double val = fma(X.K1, p0 * p12, X.K2 * (q0 * q12));
    double dval = 0;
    if (deriv) {
      const double* dBq = W.dB[q];
      const double dp0 = dBq[X.b[0]], dp1 = dBq[X.b[1]], dp2 = dBq[X.b[2]];
      const double dq0 = dBq[X.b[3]], dq1 = dBq[X.b[4]], dq2 = dBq[X.b[5]];
      const double dP = fma(dp0, p12, p0 * fma(dp1, p2, p1 * dp2));
      const double dQ = fma(dq0, q12, q0 * fma(dq1, q2, q1 * dq2));
      dval = fma(X.K1, dP, X.K2 * dQ);
    }
    CSet& C = W.cs[set[q]];
    const int d = X.dest;
    if (d < kNCV) { C.cv[d] = val; C.cvd[d] = dval; }
    else { C.w[d - kNCV] = val; C.wd[d - kNCV] = dval; }
  };
  // the qi-th time with (deriv) or without derivatives
  auto time_of = [&](int qi, bool deriv) {
    int q = 0;
    for (int qq = 0, cnt = 0; qq < nt; ++qq)
      if ((((dmask >> qq) & 1u) != 0) == deriv) { if (cnt == qi) q = qq; ++cnt; }
    return q;
  };
  const unsigned dm = dmask & ((1u << nt) - 1u);
  const int nder = __popc(dm) * nexpr, nval = nt * nexpr - nder;
  const int wd = (nder + 31) >> 5;  // warps for the derivative expressions, one per lane
  if (NW >= 4 && wd > 0 && wd < NW) {
    // derivative expressions (about three times the FP64 work of a value) on the top wd warps, one
    // per lane; the value-only expressions spread over the other warps
    if (g.wq >= NW - wd) {
      const int i = (g.wq - (NW - wd)) * 32 + g.lane;
      if (i < nder) { const int qi = i / nexpr; expr(time_of(qi, true), i - qi * nexpr, true); }
    } else {
      for (int i = g.gt; i < nval; i += 32 * (NW - wd)) { const int qi = i / nexpr; expr(time_of(qi, false), i - qi * nexpr, false); }
    }
  } else {
    for (int p = g.gt; p < nt * nexpr; p += 32 * NW) {
      const int q = p / nexpr;
      expr(q, p - q * nexpr, ((dmask >> q) & 1u) != 0);
    }
  }
  g.sync();
}

// Metric functionals of a shared-memory vector v (every warp computes them): Ψ(v) and the δρ
// sum; Φ̇ = PA·ρ + PB·v_Φ + (-ℋ)Ψ.
// Lane l < 16 holds the Ψ term of weight w[l], lane 16 + m the δρ term of weight w[16 + m]
// (kMaxFun = 16); fc is the component it reads (n, a zero entry, when the lane has no term).
template <typename T>
__device__ __forceinline__ void functionals(int fc, const T* v, const double* w, double& psi, double& rho) {
  const int lane = threadIdx.x & 31;
  double t = w[lane] * (double)v[fc];
#pragma unroll
  for (int o = 8; o; o >>= 1) t += __shfl_xor_sync(FULL, t, o);
  psi = __shfl_sync(FULL, t, 0);
  rho = __shfl_sync(FULL, t, 16);
}

__device__ __forceinline__ double phidot(const double* cv, double rho, double xphi, double psi) {
  return cv[CV_PA] * rho + cv[CV_PB] * xphi + cv[CV_MH] * psi;
}

// out = J(τ) x for the thread's components (x in shared memory, complete; x[n] == 0).
template <int NW, int NSL>
__device__ __forceinline__ void matvec(const Grp<NW>& g, const double* x, const CSet& C, const CompDesc* __restrict__ comps,
                                       const ModelDesc& M, double k, double (&out)[NSL], double* phid_out = nullptr,
                                       double* psi_out = nullptr) {
  const int gt = g.gt;
  const double* cv = C.cv;
  double psi = 0, phd = 0;
  if (g.pp || phid_out || psi_out) {  // warp-uniform: only warps with metric-coupled rows need Ψ, Φ̇
    double rho;
    functionals(g.fc, x, C.w, psi, rho);
    phd = phidot(cv, rho, x[0], psi);
  }
  if (phid_out) *phid_out = phd;
  if (psi_out) *psi_out = psi;
  const double k34 = 0.75 * k;
#pragma unroll
  for (int s = 0; s < NSL; ++s) {
    const int i = comp_of<NW>(gt, s);
    double o = 0;
    if (i < M.n) {
      const CompDesc& D = comps[i];
      o = cv[D.sp] * (D.A * x[D.ip] + D.C * x[D.inx]) + (cv[D.dg] + cv[D.tr]) * x[i];
      if (s == 0 && gt < 32) o += cv[D.e0] * x[D.e0c] + cv[D.e1] * x[D.e1c] + cv[D.e2] * x[D.e2c] + cv[D.dx] * (x[D.dxa] - k34 * x[D.dxb]);
      if ((g.pp >> s) & 1u) o += cv[D.phid] * phd + cv[D.psid] * psi;
    }
    out[s] = o;
  }
}

// out = (dJ/dτ) x
template <int NW, int NSL>
__device__ __forceinline__ void matvec_dtau(const Grp<NW>& g, const double* x, const CSet& C, const CompDesc* __restrict__ comps,
                                            const ModelDesc& M, double k, double (&out)[NSL], double* dpsi_out = nullptr) {
  const int gt = g.gt;
  double psi = 0, dpsi = 0, phd = 0, dphd = 0;
  const double* cv = C.cv; const double* cvd = C.cvd;
  if (g.pp || dpsi_out) {  // warp-uniform, as in matvec
    double rho, drho;
    functionals(g.fc, x, C.w, psi, rho);
    functionals(g.fc, x, C.wd, dpsi, drho);
    phd = phidot(cv, rho, x[0], psi);
    dphd = cvd[CV_PA] * rho + cv[CV_PA] * drho + cvd[CV_PB] * x[0] + cvd[CV_MH] * psi + cv[CV_MH] * dpsi;
  }
  if (dpsi_out) *dpsi_out = dpsi;
  const double k34 = 0.75 * k;
#pragma unroll
  for (int s = 0; s < NSL; ++s) {
    const int i = comp_of<NW>(gt, s);
    double o = 0;
    if (i < M.n) {
      const CompDesc& D = comps[i];
      o = cvd[D.sp] * (D.A * x[D.ip] + D.C * x[D.inx]) + (cvd[D.dg] + cvd[D.tr]) * x[i];
      if ((g.pp >> s) & 1u) o += cvd[D.phid] * phd + cv[D.phid] * dphd + cvd[D.psid] * psi + cv[D.psid] * dpsi;
      if (s == 0 && gt < 32) o += cvd[D.e0] * x[D.e0c] + cvd[D.e1] * x[D.e1c] + cvd[D.e2] * x[D.e2c] + cvd[D.dx] * (x[D.dxa] - k34 * x[D.dxb]);
    }
    out[s] = o;
  }
}

// out = J(τ) x and dout = (dJ/dτ) x from one read of x and one evaluation of the metric functionals
// (the accepted step's f(t1, y1) and the next step's ∂f/∂τ share the t1 coefficient set).
template <int NW, int NSL>
__device__ __forceinline__ void matvec_jd(const Grp<NW>& g, const double* x, const CSet& C, const CompDesc* __restrict__ comps,
                                          const ModelDesc& M, double k, double (&out)[NSL], double (&dout)[NSL]) {
  const int gt = g.gt;
  double psi = 0, dpsi = 0, phd = 0, dphd = 0;
  const double* cv = C.cv; const double* cvd = C.cvd;
  if (g.pp) {  // warp-uniform, as in matvec
    double rho, drho;
    functionals(g.fc, x, C.w, psi, rho);
    functionals(g.fc, x, C.wd, dpsi, drho);
    phd = phidot(cv, rho, x[0], psi);
    dphd = cvd[CV_PA] * rho + cv[CV_PA] * drho + cvd[CV_PB] * x[0] + cvd[CV_MH] * psi + cv[CV_MH] * dpsi;
  }
  const double k34 = 0.75 * k;
#pragma unroll
  for (int s = 0; s < NSL; ++s) {
    const int i = comp_of<NW>(gt, s);
    double o = 0, d = 0;
    if (i < M.n) {
      const CompDesc& D = comps[i];
      const double ax = D.A * x[D.ip] + D.C * x[D.inx], xi = x[i];
      o = cv[D.sp] * ax + (cv[D.dg] + cv[D.tr]) * xi;
      d = cvd[D.sp] * ax + (cvd[D.dg] + cvd[D.tr]) * xi;
      if (s == 0 && gt < 32) {
        const double x0 = x[D.e0c], x1 = x[D.e1c], x2 = x[D.e2c], xd = x[D.dxa] - k34 * x[D.dxb];
        o += cv[D.e0] * x0 + cv[D.e1] * x1 + cv[D.e2] * x2 + cv[D.dx] * xd;
        d += cvd[D.e0] * x0 + cvd[D.e1] * x1 + cvd[D.e2] * x2 + cvd[D.dx] * xd;
      }
      if ((g.pp >> s) & 1u) {
        o += cv[D.phid] * phd + cv[D.psid] * psi;
        d += cvd[D.phid] * phd + cv[D.phid] * dphd + cvd[D.psid] * psi + cv[D.psid] * dpsi;
      }
    }
    out[s] = o;
    dout[s] = d;
  }
}

// ------------------------------------------------------------------------------------------
// structured factorisation of M = s I - B and its solves
//
// Chains of at most 32 rows are eliminated with warp scans (lane j holds row last - j): the
// forward elimination c_i = r_i - m_i c_{i+1} runs up the lanes, the back substitution
// z_i = d_i c_i - d_i b_i z_{i-1} down the lanes; both are affine recurrences whose Kogge-Stone
// multipliers depend only on the factorisation and are tabulated per row (fA, bA, bP) once per
// step.  The back substitution is run with a zero head value; the head value h enters linearly as
// z_i += P_i h (P_i = bP[i]), which the consumers of a solution add for their own rows.  A solve is
// then one scan phase (both directions), one head phase and two barriers.  Longer chains fall
// back to one thread per chain with an exact back substitution.  The 8x8 head is inverted explicitly
// (Gauss-Jordan with partial pivoting, one row per lane), so a head solve is an 8-term product.
__device__ __forceinline__ int head_local(int i) { return (i >= 3 && i <= 10) ? i - 3 : -1; }

template <typename ST>
struct Factor {
  ST is, ihc;
  ST S00, S01, S10, S11;  // inverse of I - Vᵀ M⁻¹ U
};

template <typename T>
__device__ __forceinline__ T shfl_up_(T v, int d) { return __shfl_up_sync(FULL, v, d); }

// chains (2p, 2p+1) for pass p; lane j holds row last - j (forward) or first + j (back)
struct ChainPair {
  int f0, l0, a0, f1, l1, a1;  // first, last, attach (a = -2: absent chain)
};
__device__ __forceinline__ ChainPair chain_pair(const ModelDesc& M, int p) {
  ChainPair c;
  const int c0 = 2 * p, c1 = 2 * p + 1;
  c.f0 = M.chFirst[c0]; c.l0 = M.chLast[c0]; c.a0 = M.chAttach[c0];
  if (c1 < M.nchain) { c.f1 = M.chFirst[c1]; c.l1 = M.chLast[c1]; c.a1 = M.chAttach[c1]; }
  else { c.f1 = 0; c.l1 = -1; c.a1 = -2; }
  return c;
}

// M⁻¹ applied in place to NV vectors (input complete; ends with a group barrier).
template <int NV, int NW, int NSL, typename ST>
__device__ __forceinline__ void solve_M(const Grp<NW>& g, ModeMem<NW, NSL, ST>& W, const ModelDesc& M, const Factor<ST>& F,
                                        bool scan, ST* v0, ST* v1) {
  const int gt = g.gt, lane = g.lane;
  const int npair = (M.nchain + 1) >> 1;
  // forward elimination along the chains, truncation end first
  if (scan) {
    for (int p = g.wq; p < npair; p += NW) {
      const ChainPair c = chain_pair(M, p);
      const int i0 = c.l0 - lane, i1 = c.l1 - lane;
      const bool on0 = i0 >= c.f0, on1 = i1 >= c.f1;
      // every load unconditional from a row inside the arrays (off-chain lanes read row 0), then
      // zeroed by a select: no branch around the loads
      const int j0 = on0 ? i0 : 0, j1 = on1 ? i1 : 0;
      ST m0[5], m1[5], n0[5], n1[5];
#pragma unroll
      for (int q = 0; q < 5; ++q) {
        const ST a0 = W.fA[q][j0], a1 = W.fA[q][j1], b0 = W.bA[q][j0], b1 = W.bA[q][j1];
        m0[q] = on0 ? a0 : ST(0); m1[q] = on1 ? a1 : ST(0);
        n0[q] = on0 ? b0 : ST(0); n1[q] = on1 ? b1 : ST(0);
      }
      const ST e0 = W.dinv[j0], e1 = W.dinv[j1], r0 = v0[j0], r1 = v0[j1];
      const ST d0 = on0 ? e0 : ST(0), d1 = on1 ? e1 : ST(0);
      ST x0 = on0 ? r0 : ST(0), x1 = on1 ? r1 : ST(0);
      ST y0 = ST(0), y1 = ST(0);
      if (NV > 1) { const ST s0 = v1[j0], s1 = v1[j1]; y0 = on0 ? s0 : ST(0); y1 = on1 ? s1 : ST(0); }
#pragma unroll
      for (int q = 0; q < 5; ++q) {  // forward elimination, up the lanes
        const int d = 1 << q;
        const ST px0 = shfl_up_(x0, d), px1 = shfl_up_(x1, d);
        x0 += m0[q] * px0; x1 += m1[q] * px1;
        if (NV > 1) { const ST py0 = shfl_up_(y0, d), py1 = shfl_up_(y1, d); y0 += m0[q] * py0; y1 += m1[q] * py1; }
      }
      if (i0 == c.f0 && c.a0 >= 0) { W.cf[0][2 * p] = x0; if (NV > 1) W.cf[1][2 * p] = y0; }
      if (i1 == c.f1 && c.a1 >= 0) { W.cf[0][2 * p + 1] = x1; if (NV > 1) W.cf[1][2 * p + 1] = y1; }
      x0 *= d0; x1 *= d1;
      if (NV > 1) { y0 *= d0; y1 *= d1; }
#pragma unroll
      for (int q = 0; q < 5; ++q) {  // back substitution with a zero head value, down the lanes
        const int d = 1 << q;
        const ST px0 = __shfl_down_sync(FULL, x0, d), px1 = __shfl_down_sync(FULL, x1, d);
        x0 += n0[q] * px0; x1 += n1[q] * px1;
        if (NV > 1) {
          const ST py0 = __shfl_down_sync(FULL, y0, d), py1 = __shfl_down_sync(FULL, y1, d);
          y0 += n0[q] * py0; y1 += n1[q] * py1;
        }
      }
      if (on0) { v0[i0] = x0; if (NV > 1) v1[i0] = y0; }
      if (on1) { v0[i1] = x1; if (NV > 1) v1[i1] = y1; }
    }
    if (g.wq == NW - 1 && (lane == 16 || lane == 17)) {  // CDM: [[s, 1], [0, s+ℋ]]
      ST* v = lane == 16 ? v0 : v1;
      if (lane == 16 || NV > 1) {
        const ST zt = v[2] * F.ihc;
        v[2] = zt;
        v[1] = (v[1] - zt) * F.is;
      }
    } else if (g.wq == NW - 1 && lane == 18) {
      v0[0] *= F.is;
      if (NV > 1) v1[0] *= F.is;
    }
    // 8x8 head with the chains' couplings: explicit inverse.  When every chain attached to the
    // head is in pair 0 (the photon T and P tails), warp 0 has just eliminated them itself and
    // solves the head at once, without waiting for the other warps' chains.
    if (W.hfused) {
      if (g.wq == 0) __syncwarp();
    } else {
      g.sync();
    }
    if (g.wq == 0 && lane < 8) {
      const int ch = W.hatt[lane];
      ST b0 = v0[3 + lane], b1 = NV > 1 ? v1[3 + lane] : ST(0);
      if (ch >= 0) { const ST hm = W.hmul[ch]; b0 -= hm * W.cf[0][ch]; if (NV > 1) b1 -= hm * W.cf[1][ch]; }
      ST o0 = 0, o1 = 0;
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const ST hq = W.Hinv[lane * 8 + q];
        o0 += hq * __shfl_sync(0xffu, b0, q);
        if (NV > 1) o1 += hq * __shfl_sync(0xffu, b1, q);
      }
      v0[3 + lane] = o0;
      if (NV > 1) v1[3 + lane] = o1;
    }
    g.sync();
    return;
  } else {
    for (int ch = gt; ch < M.nchain; ch += 32 * NW) {
      const int first = M.chFirst[ch], last = M.chLast[ch];
      ST c0 = v0[last], c1 = NV > 1 ? v1[last] : ST(0);
      for (int i = last - 1; i >= first; --i) {
        const ST m = W.mfw[i];
        c0 = v0[i] - m * c0; v0[i] = c0;
        if (NV > 1) { c1 = v1[i] - m * c1; v1[i] = c1; }
      }
      const int at = M.chAttach[ch];
      if (at >= 0) { const ST hm = W.hmul[ch]; v0[at] -= hm * c0; if (NV > 1) v1[at] -= hm * c1; }
    }
  }
  g.sync();
  if (g.wq == 0) {
    if (lane < 8) {  // 8x8 head: explicit inverse
      ST o0 = 0, o1 = 0;
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const ST hq = W.Hinv[lane * 8 + q];
        o0 += hq * v0[3 + q];
        if (NV > 1) o1 += hq * v1[3 + q];
      }
      __syncwarp(0xffu);
      v0[3 + lane] = o0;
      if (NV > 1) v1[3 + lane] = o1;
    } else if (lane == 8 || lane == 9) {  // CDM: [[s, 1], [0, s+ℋ]]
      ST* v = lane == 8 ? v0 : v1;
      if (lane == 8 || NV > 1) {
        const ST zt = v[2] * F.ihc;
        v[2] = zt;
        v[1] = (v[1] - zt) * F.is;
      }
    } else if (lane == 10) {
      v0[0] *= F.is;
      if (NV > 1) v1[0] *= F.is;
    }
  }
  g.sync();
  // back substitution away from the head (one thread per chain)
  {
    for (int ch = gt; ch < M.nchain; ch += 32 * NW) {
      const int first = M.chFirst[ch], last = M.chLast[ch], at = M.chAttach[ch];
      ST z0 = at >= 0 ? v0[at] : ST(0), z1 = (NV > 1 && at >= 0) ? v1[at] : ST(0);
      for (int i = first; i <= last; ++i) {
        const ST sb = W.sub[i], di = W.dinv[i];
        z0 = (v0[i] - sb * z0) * di; v0[i] = z0;
        if (NV > 1) { z1 = (v1[i] - sb * z1) * di; v1[i] = z1; }
      }
    }
  }
  g.sync();
}

// Functionals in solve precision from the factorisation's weight copy: Ψ(v), δρ sum, Φ̇.
template <int NW, int NSL, typename ST>
__device__ __forceinline__ void functionals_st(const Grp<NW>& g, const ModeMem<NW, NSL, ST>& W, const ST* v, ST& psi, ST& phd) {
  const int lane = threadIdx.x & 31;
  ST t = W.wS[lane] * v[g.fc];
#pragma unroll
  for (int o = 8; o; o >>= 1) t += __shfl_xor_sync(FULL, t, o);
  psi = __shfl_sync(FULL, t, 0);
  const ST rho = __shfl_sync(FULL, t, 16);
  phd = W.fS[0] * rho + W.fS[1] * v[0] + W.fS[2] * psi;
}

template <int NW, int NSL, typename ST>
__device__ __forceinline__ void factorize(const Grp<NW>& g, ModeMem<NW, NSL, ST>& W, Factor<ST>& F, const CSet& C,
                                          const CompDesc* __restrict__ comps, const ModelDesc& M, double k, double h,
                                          double s, double gam, bool scan) {
  const int gt = g.gt, lane = g.lane;
  const double* cv = C.cv;
  // per-row inputs, all threads: diagonal s - (dg + tr), the two chain couplings, the rank-2
  // columns; the functional weights in solve precision
#pragma unroll
  for (int sl = 0; sl < NSL; ++sl) {
    const int i = comp_of<NW>(gt, sl);
    if (i < M.n) {
      const CompDesc& D = comps[i];
      const double spv = cv[D.sp];
      W.dd[i] = to_st<ST>(s - (cv[D.dg] + cv[D.tr]));
      W.sup[i] = to_st<ST>(-spv * D.C);
      W.sub[i] = to_st<ST>(-spv * D.A);
      W.Z1[i] = to_st<ST>(cv[D.phid]);
      W.Z2[i] = to_st<ST>(cv[D.psid]);
    }
  }
  for (int q = gt; q < kWF; q += 32 * NW) W.wS[q] = to_st<ST>(C.w[q]);
  if (gt < 3) W.fS[gt] = to_st<ST>(cv[gt == 0 ? CV_PA : gt == 1 ? CV_PB : CV_MH]);
  g.sync();
  for (int ch = gt; ch < M.nchain; ch += 32 * NW) {  // chain LU from the truncation end (precision ST)
    const int first = M.chFirst[ch], last = M.chLast[ch], at = M.chAttach[ch];
    ST dn = rcp<ST>(W.dd[last]);
    W.dinv[last] = dn; W.mfw[last] = 0;
    for (int i = last - 1; i >= first; --i) {
      const ST sp = W.sup[i];
      const ST di = rcp<ST>(W.dd[i] - sp * W.sub[i + 1] * dn);
      W.dinv[i] = di; W.mfw[i] = sp * dn;
      dn = di;
    }
    if (at >= 0) {
      const CompDesc& D = comps[at];
      const ST hs = to_st<ST>(-cv[D.sp] * D.C);  // coefficient of x[first] in the head row
      const ST hm = hs * dn;
      W.hmul[ch] = hm;
      W.hcorr[ch] = hm * W.sub[first];
    }
  }
  if (g.wq == NW - 1 && lane >= 16 && lane < 24) {  // assemble head row 3 + j
    const int j = lane - 16, r = 3 + j;
    const double k34 = 0.75 * k;
    const CompDesc& D = comps[r];
    double row[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) row[c] = 0;
    row[j] += s - (cv[D.dg] + cv[D.tr]);
    const double spv = cv[D.sp];
    int c;
    if ((c = head_local(D.ip)) >= 0) row[c] -= spv * D.A;
    if ((c = head_local(D.inx)) >= 0) row[c] -= spv * D.C;
    if ((c = head_local(D.e0c)) >= 0) row[c] -= cv[D.e0];
    if ((c = head_local(D.e1c)) >= 0) row[c] -= cv[D.e1];
    if ((c = head_local(D.e2c)) >= 0) row[c] -= cv[D.e2];
    if ((c = head_local(D.dxa)) >= 0) row[c] -= cv[D.dx];
    if ((c = head_local(D.dxb)) >= 0) row[c] += k34 * cv[D.dx];
#pragma unroll
    for (int q = 0; q < 8; ++q) W.H[j * 8 + q] = to_st<ST>(row[q]);
  }
  g.sync();
  const int npair = (M.nchain + 1) >> 1;
  if (scan) {
    // Kogge-Stone multipliers of both chain recurrences, one chain row per lane; with several
    // warps, warp 0 is left to the head inversion below
    constexpr int w0 = NW > 1 ? 1 : 0, nwp = NW > 1 ? NW - 1 : 1;
    for (int p = g.wq - w0; p >= 0 && p < npair; p += nwp) {
#pragma unroll
      for (int hc = 0; hc < 2; ++hc) {
        const int ch = 2 * p + hc;
        const bool live = ch < M.nchain;
        const int first = live ? M.chFirst[ch] : 0, last = live ? M.chLast[ch] : -1;
        {  // forward: lane j = row last - j, element (a_j = -m_j, c_j); a_0 = 0
          const int i = last - lane;
          const bool on = i >= first;
          ST a = (on && lane > 0) ? -W.mfw[i] : ST(0);
#pragma unroll
          for (int q = 0; q < 5; ++q) {
            const int d = 1 << q;
            const ST ap = shfl_up_(a, d);
            if (on) W.fA[q][i] = lane >= d ? a : ST(0);
            if (lane >= d) a *= ap;
          }
        }
        {  // back: lane j = row last - j, element (a_j = -d_j b_j, d_j c_j); the head value
           // follows the last lane (row first), so the scan runs down the lanes
          const int i = last - lane, L = last - first + 1;
          const bool on = i >= first;
          ST a = on ? -W.dinv[i] * W.sub[i] : ST(0);
#pragma unroll
          for (int q = 0; q < 5; ++q) {
            const int d = 1 << q;
            const ST ap = __shfl_down_sync(FULL, a, d);
            const bool in = lane + d < L;
            if (on) W.bA[q][i] = in ? a : ST(0);
            if (in) a *= ap;
          }
          if (on) W.bP[i] = a;  // ∂z_i/∂h
        }
      }
    }
  }
  if (g.wq == 0) {
    // head inverse: Gauss-Jordan with partial pivoting on [H | I], lane q (mod 16) holding column q
    // in registers, so the pivot search is lane kk's own register scan and a pivot step moves only
    // the pivot row index, the pivot and the eliminated column's multipliers between lanes
    const int q = lane & 15;
    ST col[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) col[r] = q < 8 ? W.H[r * 8 + q] : ST(r == q - 8 ? 1 : 0);
    if (q == 4) col[4] -= W.hcorr[0];  // F2 (Schur complement of the F tail)
    if (q == 7) col[7] -= W.hcorr[1];  // G2 (G tail)
#pragma unroll
    for (int kk = 0; kk < 8; ++kk) {
      int p = kk;  // first row of largest magnitude at or below kk (meaningful on lane kk)
      ST best = fabs(col[kk]);
#pragma unroll
      for (int r = kk + 1; r < 8; ++r) { const ST v = fabs(col[r]); if (v > best) { best = v; p = r; } }
      p = __shfl_sync(FULL, p, kk);
      ST vp = col[kk];
#pragma unroll
      for (int r = kk + 1; r < 8; ++r) if (r == p) { vp = col[r]; col[r] = col[kk]; }
      col[kk] = vp;
      ST m[8];
#pragma unroll
      for (int r = 0; r < 8; ++r) m[r] = __shfl_sync(FULL, col[r], kk);  // column kk after the swap
      const ST ip = rcp<ST>(m[kk]);
      col[kk] *= ip;
#pragma unroll
      for (int r = 0; r < 8; ++r) if (r != kk) col[r] -= m[r] * col[kk];
    }
    if (lane >= 8 && lane < 16) {
#pragma unroll
      for (int r = 0; r < 8; ++r) W.Hinv[r * 8 + (lane - 8)] = col[r];
    }
  }
  F.is = to_st<ST>(h * gam);
  F.ihc = rcp<ST>(to_st<ST>(s - cv[CV_MH]));
  g.sync();
  // rank-2 correction: Z1 = M⁻¹ c_Φ̇, Z2 = M⁻¹ c_Ψ
  solve_M<2>(g, W, M, F, scan, W.Z1, W.Z2);
#pragma unroll
  for (int sl = 0; sl < NSL; ++sl) {  // head-value terms of the chain back substitutions (own rows)
    const int i = comp_of<NW>(gt, sl);
    if (i < M.n && W.att[i] >= 0) { const ST P = W.bP[i]; W.Z1[i] += P * W.Z1[W.att[i]]; W.Z2[i] += P * W.Z2[W.att[i]]; }
  }
  ST psi1, p1, psi2, p2;
  functionals_st(g, W, W.Z1, psi1, p1);
  functionals_st(g, W, W.Z2, psi2, p2);
  const ST a = 1 - p1, b = -p2, c = -psi1, d = 1 - psi2;
  const ST idet = ST(1) / (a * d - b * c);
  F.S00 = d * idet; F.S01 = -b * idet; F.S10 = -c * idet; F.S11 = a * idet;
}

// u = W⁻¹ W.r for the thread's own components, in registers (W.r complete on entry; W.r is
// overwritten; no barrier follows).
template <int NW, int NSL, typename ST>
__device__ __forceinline__ void solve_W(const Grp<NW>& g, ModeMem<NW, NSL, ST>& W, const Factor<ST>& F, const ModelDesc& M,
                                        bool scan, ST (&u)[NSL]) {
  solve_M<1>(g, W, M, F, scan, W.r, W.r);
  ST psi, ph;
  functionals_st(g, W, W.r, psi, ph);
  const ST t0 = F.S00 * ph + F.S01 * psi, t1 = F.S10 * ph + F.S11 * psi;
#pragma unroll
  for (int sl = 0; sl < NSL; ++sl) {
    const int i = comp_of<NW>(g.gt, sl);
    const int ic = i < M.n ? i : 0;
    const int at = W.att[ic];
    const ST ri = W.r[ic], ra = W.r[at >= 0 ? at : ic], P = W.bP[ic], z1 = W.Z1[ic], z2 = W.Z2[ic];
    const ST rh = at >= 0 ? ri + P * ra : ri;  // head-value term of the chain back substitution
    u[sl] = i < M.n ? rh + z1 * t0 + z2 * t1 : ST(0);
  }
}

// U = W⁻¹ b with FP64 iterative refinement (W = s I - J at the step start): up to `refine`
// corrections, stopping once the largest correction is below 1e-3 in units of the integrator's
// error weights (isk = 1/(atol + rtol |y|)).  In the stiff tight-coupling era the FP32 head solve
// has condition number ~κ̇h and one correction leaves a bias that accumulates over the steps;
// elsewhere one correction is enough.  W.r and W.x must be free (no thread still reading them) on
// entry.
template <int NW, int NSL, typename ST>
__device__ __forceinline__ void stage_solve(const Grp<NW>& g, ModeMem<NW, NSL, ST>& W, const Factor<ST>& F, const CSet& CJ,
                            const CompDesc* __restrict__ comps, const ModelDesc& M, double k, double s, int refine,
                            bool scan, const float (&isk)[NSL], const double (&b)[NSL], double (&U)[NSL],
                            float* first_correction = nullptr) {
  const int gt = g.gt;
#pragma unroll
  for (int sl = 0; sl < NSL; ++sl) { const int i = comp_of<NW>(gt, sl); if (i < M.n) W.r[i] = to_st<ST>(b[sl]); }
  // one loop over the solve and its corrections, so the structured solve's code appears once
  for (int it = 0;; ++it) {
    g.sync();
    ST u[NSL];
    solve_W(g, W, F, M, scan, u);
    if (it == 0) {
#pragma unroll
      for (int sl = 0; sl < NSL; ++sl) U[sl] = from_st(u[sl]);
    } else {
      float c = 0.0f;
#pragma unroll
      for (int sl = 0; sl < NSL; ++sl) {
        const int i = comp_of<NW>(gt, sl);
        if (i < M.n) { const ST d = u[sl]; U[sl] += from_st(d); c = fmaxf(c, fabsf((float)d) * isk[sl]); }
      }
      const int r = it - 1;  // correction index
      if (r + 1 < refine || (r == 0 && first_correction)) {
        const float cm = group_max(g, W, c);
        if (r == 0 && first_correction) *first_correction = cm;
        if (r + 1 < refine && cm < 1e-3f) break;
      }
    }
    if (it >= refine) break;
    // residual b - W U in FP64 for the next correction
#pragma unroll
    for (int sl = 0; sl < NSL; ++sl) { const int i = comp_of<NW>(gt, sl); if (i < M.n) W.x[i] = U[sl]; }
    g.sync();
    double JU[NSL];
    matvec<NW, NSL>(g, W.x, CJ, comps, M, k, JU);
#pragma unroll
    for (int sl = 0; sl < NSL; ++sl) {
      const int i = comp_of<NW>(gt, sl);
      if (i < M.n) W.r[i] = to_st<ST>(b[sl] - (s * U[sl] - JU[sl]));  // s U - J U ≈ b first: rounding of order ε|b|, not ε|J U|
    }
  }
}

// ------------------------------------------------------------------------------------------
// outputs at one saved time τ for state y (coefficient set kNSets-1 is used as scratch)
template <int NW, int NSL, typename ST>
__device__ void emit_output(const Grp<NW>& g, ModeMem<NW, NSL, ST>& W, const PtArgs& A, const CosmoDesc* cd,
                            const double* tab, const CompDesc* __restrict__ comps, const ModelDesc& M, const ModeK& mk,
                            double tau, const double (&y)[NSL], int item, int j) {
  const int gt = g.gt;
  if (A.output == SBZ_OUT_STATE) {
    double* o = A.out + ((size_t)item * A.ntau + j) * M.n;
#pragma unroll
    for (int sl = 0; sl < NSL; ++sl) { const int i = comp_of<NW>(gt, sl); if (i < M.n) o[i] = y[sl]; }
    return;
  }
  if (A.output != SBZ_OUT_SOURCES && A.output != SBZ_OUT_SOURCES4 && A.output != SBZ_OUT_FACTORS) return;
  // line-of-sight sources (src/models/cosmologies.jl:99-105)
  const int so = kNSets - 1;
  const double k = mk.k;
  coef_eval(g, W, &so, &tau, 1, 1u, true, cd, tab, M.nexpr, M.nx, mk);
  const CSet& CS = W.cs[so];
#pragma unroll
  for (int sl = 0; sl < NSL; ++sl) { const int i = comp_of<NW>(gt, sl); if (i < M.n) W.x[i] = y[sl]; }
  g.sync();
  double fy[NSL], dJy[NSL], Jf[NSL], phid, psi, dpsi_w, psi_f;
  matvec<NW, NSL>(g, W.x, CS, comps, M, k, fy, &phid, &psi);
  matvec_dtau<NW, NSL>(g, W.x, CS, comps, M, k, dJy, &dpsi_w);
#pragma unroll
  for (int sl = 0; sl < NSL; ++sl) { const int i = comp_of<NW>(gt, sl); if (i < M.n) W.f[i] = fy[sl]; }
  g.sync();
  matvec<NW, NSL>(g, W.f, CS, comps, M, k, Jf, nullptr, &psi_f);
  if (g.wq == 0) {
    // second derivative of Π = F2 + G0 + G2 along the flow: (J'y + J f) restricted to those rows
    double gv = 0;
    if (gt == 7 || gt == 8 || gt == 10) gv = dJy[0] + Jf[0];
    const double Pidd = warp_sum(gv);
    if (gt == 0) {
      const double ek = W.src[0], kdd = W.src[1], kddd = W.src[2];
      const double kd = W.B[0][B_KD];
      const double v = -kd * ek, vd = (kd * kd - kdd) * ek, vdd = (-kd * kd * kd + 3 * kd * kdd - kddd) * ek;
      const double Pi = W.x[7] + W.x[8] + W.x[10];
      const double Pid = W.f[7] + W.f[8] + W.f[10];
      const double psid = dpsi_w + psi_f;  // Ψ' = (∂Ψ/∂τ) y + Ψ(f)
      const double sSW = v * (W.x[5] * 0.25 + psi + Pi / 16), sISW = ek * (psid + phid);
      const double sDop = (vd * W.x[4] + v * W.f[4]) * mk.ik2;
      const double sPol = 3.0 / 16.0 * mk.ik2 * (vdd * Pi + 2 * vd * Pid + v * Pidd);
      const double chi = cd->tau0 - tau;
      const double SE = 3.0 / 16.0 * v * Pi / ((k * chi) * (k * chi));
      if (A.output == SBZ_OUT_FACTORS) {
        double* o = A.out + ((size_t)item * A.ntau + j) * 7;
        o[0] = W.x[5] * 0.25 + psi + Pi / 16; o[1] = psid + phid; o[2] = W.x[4]; o[3] = W.f[4];
        o[4] = Pi; o[5] = Pid; o[6] = Pidd;
      } else if (A.output == SBZ_OUT_SOURCES4) {
        double* o = A.out + ((size_t)item * A.ntau + j) * 4;
        o[0] = k * (sSW + sISW); o[1] = k * sDop; o[2] = k * sPol; o[3] = k * k * SE;
      } else {
        const double Spsi = (tau >= cd->taurec) ? -(psi + W.x[0]) * (tau - cd->taurec) / (cd->tau0 - cd->taurec) / chi : 0.0;
        double* o = A.out + ((size_t)item * A.ntau + j) * 3;
        o[0] = k * (sSW + sISW + sDop + sPol); o[1] = k * k * SE; o[2] = Spsi;
      }
    }
  }
  g.sync();
}

template <int NW, int NSL, typename ST>
__device__ void pt_body(const PtArgs& A, const ModelDesc& M, const CompDesc* __restrict__ comps, ModeMem<NW, NSL, ST>& W,
                        const Grp<NW>& g) {
  constexpr int NT = 32 * NW;
  const int gt = g.gt;
  const int n = M.n;
  for (int i = gt; i < kNSets * (int)(sizeof(CSet) / sizeof(double)); i += NT) reinterpret_cast<double*>(W.cs)[i] = 0;
  for (int i = n + gt; i <= NT * NSL; i += NT) { W.x[i] = 0; W.f[i] = 0; W.r[i] = 0; W.Z1[i] = 0; W.Z2[i] = 0; }
  g.sync();
  const double rtol = A.rtol, atol = A.atol;
  const double inv_n = 1.0 / n;
  bool scan = true;  // every chain fits a warp scan
  for (int c = 0; c < M.nchain; ++c) scan = scan && (M.chLast[c] - M.chFirst[c] < 32);
  for (int i = gt; i < NT * NSL; i += NT) {
    int at = -1;
    for (int c = 0; c < M.nchain; ++c) if (scan && i >= M.chFirst[c] && i <= M.chLast[c]) at = M.chAttach[c];
    W.att[i] = (int16_t)at;
  }
  if (gt < 8) {
    int hc = -1;
    for (int c = 0; c < M.nchain; ++c) if (M.chAttach[c] == 3 + gt) hc = c;
    W.hatt[gt] = hc;
  }
  if (gt == 0) {
    bool f = scan;
    for (int c = 0; c < M.nchain; ++c) if (M.chAttach[c] >= 0 && c > 1) f = false;
    W.hfused = f ? 1 : 0;
  }

  for (;;) {
    if (gt == 0) W.item = (int)atomicAdd(A.counter, 1u);
    g.sync();
    const int slot = W.item;
    g.sync();  // every thread has read the slot before the next mode overwrites it
    if (slot >= A.nitems) break;
    const int item = A.order ? A.order[slot] : slot;
    const int c = A.item_cosmo ? A.item_cosmo[item] : 0;
    {
      const int* src = reinterpret_cast<const int*>(A.cosmos + c);
      int* dst = reinterpret_cast<int*>(&W.cdesc);
      for (int q = gt; q < (int)(sizeof(CosmoDesc) / 4); q += NT) dst[q] = src[q];
    }
    g.sync();
    const CosmoDesc* cd = &W.cdesc;
    const double* tab = A.tables + (size_t)c * A.table_stride;
    const double* taus = A.taus ? A.taus + (size_t)c * A.ntau : nullptr;
    ModeK mk;
    mk.k = A.item_k[item]; mk.k2 = mk.k * mk.k; mk.ik = 1.0 / mk.k; mk.ik2 = mk.ik * mk.ik;
    const double k = mk.k;
    const double tend = cd->tau0;
    double t = fmin(fmax(A.item_tau_ini[item], cd->tau_start), tend);
    int status = SBZ_OK;
    int64_t nacc = 0, nrej = 0;
    double y[NSL], f0[NSL], ft[NSL];
    int sJ = 0, sE = TB::NTIME;  // coefficient-set roles: J (step start) and step end swap on acceptance
    const int sIC = kNSets - 1;

    // ---- adiabatic initial conditions (src/models/cosmologies.jl:74-77 and species ieqs) ----
    coef_eval(g, W, &sIC, &t, 1, 0u, false, cd, tab, M.nexpr, M.nx, mk);
    {
      const double kdv = W.B[0][B_KD];
      double Ir = 0;
      if (g.lane < M.nx) Ir = cd->Wq[g.lane] * W.B[0][B_E + g.lane];
      Ir = warp_sum(Ir);
      const double rg = cd->Og0, rn = cd->On0 + cd->wh * Ir;  // × a⁻⁴
      const double fnu = rn / (rg + rn);
      const double Psi = 10.0 / (15.0 + 4.0 * fnu);
      const double kt = k * t;
      const double F1 = 2.0 / 3.0 * kt * Psi;
      const double F2 = -8.0 / 15.0 * k / kdv * F1;
      const double G2 = F2 / 16.0;
      const double N2 = 2.0 / 15.0 * kt * kt * Psi;
#pragma unroll
      for (int sl = 0; sl < NSL; ++sl) {
        const int i = comp_of<NW>(gt, sl);
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
            const int jb = (i - M.oH) / (M.Lh + 1), l = (i - M.oH) - jb * (M.Lh + 1);
            const double dl = cd->dlnf[jb];
            if (l == 0) v = 0.5 * Psi * dl;
            else if (l == 1) v = -1.0 / 3.0 * W.B[0][B_IQ + jb] * (0.5 * kt * Psi) * dl;
            else if (l == 2) v = -0.5 * (1.0 / 15.0 * kt * kt * Psi) * dl;
          }
        }
        y[sl] = v;
        if (i < n) W.x[i] = v;
      }
      g.sync();
      // Φ from k²(Φ - Ψ) = 12πa²Π with the initial shears: Ψ(y) is linear with unit weight on Φ
      double psi0, rho0;
      functionals(g.fc, W.x, W.cs[sIC].w, psi0, rho0);  // Φ slot still 0
      g.sync();
      if (gt == 0) { y[0] = Psi - psi0; W.x[0] = y[0]; }
      g.sync();
    }
    // outputs at or before the initial time
    int jout = 0;
    if (taus) {
      while (jout < A.ntau && taus[jout] <= t) {
        if (taus[jout] < t) {  // before the mode starts: zero
          if (A.output == SBZ_OUT_SOURCES && gt < 3) A.out[((size_t)item * A.ntau + jout) * 3 + gt] = 0;
        if (A.output == SBZ_OUT_SOURCES4 && gt < 4) A.out[((size_t)item * A.ntau + jout) * 4 + gt] = 0;
        if (A.output == SBZ_OUT_FACTORS && gt < 7) A.out[((size_t)item * A.ntau + jout) * 7 + gt] = 0;
          if (A.output == SBZ_OUT_SOURCES4 && gt < 4) A.out[((size_t)item * A.ntau + jout) * 4 + gt] = 0;
        if (A.output == SBZ_OUT_FACTORS && gt < 7) A.out[((size_t)item * A.ntau + jout) * 7 + gt] = 0;
          if (A.output == SBZ_OUT_FACTORS && gt < 7) A.out[((size_t)item * A.ntau + jout) * 7 + gt] = 0;
          if (A.output == SBZ_OUT_STATE) for (int i = gt; i < n; i += NT) A.out[((size_t)item * A.ntau + jout) * n + i] = 0;
        } else {
          emit_output(g, W, A, cd, tab, comps, M, mk, t, y, item, jout);
        }
        ++jout;
      }
    }

    // ---- integration ----
    if (t < tend) {
      coef_eval(g, W, &sJ, &t, 1, 1u, false, cd, tab, M.nexpr, M.nx, mk);
#pragma unroll
      for (int sl = 0; sl < NSL; ++sl) { const int i = comp_of<NW>(gt, sl); if (i < n) W.x[i] = y[sl]; }
      g.sync();
      matvec_jd<NW, NSL>(g, W.x, W.cs[sJ], comps, M, k, f0, ft);  // f(t, y) and ∂f/∂τ
      // initial step (Hairer-Nørsett-Wanner II.4)
      double h;
      {
        double d0 = 0, d1 = 0;
#pragma unroll
        for (int sl = 0; sl < NSL; ++sl) {
          const int i = comp_of<NW>(gt, sl);
          if (i < n) { const double sk = atol + fabs(y[sl]) * rtol; d0 += (y[sl] / sk) * (y[sl] / sk); d1 += (f0[sl] / sk) * (f0[sl] / sk); }
        }
        d0 = sqrt(group_sum(g, W, d0) * inv_n); d1 = sqrt(group_sum(g, W, d1) * inv_n);
        double h0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * d0 / d1;
        h0 = fmin(h0, tend - t);
#pragma unroll
        for (int sl = 0; sl < NSL; ++sl) { const int i = comp_of<NW>(gt, sl); if (i < n) W.x[i] = y[sl] + h0 * f0[sl]; }
        const double th = t + h0;
        coef_eval(g, W, &sE, &th, 1, 0u, false, cd, tab, M.nexpr, M.nx, mk);
        double f1[NSL];
        matvec<NW, NSL>(g, W.x, W.cs[sE], comps, M, k, f1);
        double d2 = 0;
#pragma unroll
        for (int sl = 0; sl < NSL; ++sl) {
          const int i = comp_of<NW>(gt, sl);
          if (i < n) { const double sk = atol + fabs(y[sl]) * rtol; const double q = (f1[sl] - f0[sl]) / (h0 * sk); d2 += q * q; }
        }
        d2 = sqrt(group_sum(g, W, d2) * inv_n);
        const double mx = fmax(d1, d2);
        const double h1 = (mx <= 1e-15 || !isfinite(mx)) ? fmax(1e-6, 1e-3 * h0) : pow(0.01 / mx, 0.2);
        h = fmin(100 * h0, h1);
        if (!isfinite(h) || h <= 0) h = 1e-6 * fmax(1.0, t);
      }
      constexpr double kLogErrFloor = -9.210340371976184;  // log(1e-4): the controller's floor on errold
      double lerrold = kLogErrFloor;  // log of the previous accepted error norm (controller warp)
      bool rejected = false, nonfinite = false;
      Factor<ST> F;
      int64_t iters = 0;
      // Step control runs on one warp (warp 1: no metric functionals in its operator products) while
      // the others finish the step; the loop-top barrier publishes it: the proposed size clamped to
      // the end point, 1/h, 1/(hγ), the step end and the stage times (FP64; every warp reads them).
      const int cw = NW > 1 ? 1 : 0;
      auto publish = [&](double hp, double tc) {
        const bool done = !(tc < tend);
        if (tc + 1.01 * hp >= tend) hp = tend - tc;
        const double te = (hp == tend - tc) ? tend : tc + hp;
        const bool tiny = !(hp > 1e-14 * tc);
        if (g.lane == 0) {
          W.ctlf = (done ? 1 : 0) | (tiny ? 2 : 0);
          // 1/(hγ) divided as the oracle divides it: the FP64 refinement residuals use it, and a last-bit
          // difference can move an accept/reject decision at the tolerance edge
          W.ctl[0] = hp; W.ctl[1] = 1.0 / hp; W.ctl[2] = 1.0 / (hp * TB::gam); W.ctl[3] = te;
#pragma unroll
          for (int q = 1; q < TB::NTIME; ++q) {
            int st = 1;
#pragma unroll
            for (int i = 1; i < TB::S; ++i) if (TB::tslot(i) == q) st = i;
            W.ctl[4 + q - 1] = tc + TB::c(st) * hp;
          }
          W.ctl[4 + TB::NTIME - 1] = te;
        }
      };
      if (g.wq == cw) publish(h, t);
      for (;;) {
        g.sync();  // step control published; the previous step's readers of x and the coefficient sets are done
        const int fl = W.ctlf;  // bit 0: t reached the end; bit 1: the step is below 1e-14 t
        if (fl & 1) break;
        if (++iters > A.maxiters) { status = SBZ_MAXITERS; break; }
        if (fl & 2) { status = nonfinite ? SBZ_NONFINITE : SBZ_DTMIN; break; }
        h = W.ctl[0];
        const CSet& CJ = W.cs[sJ];
        const double ih = W.ctl[1], s = W.ctl[2], tn = W.ctl[3];
        // coefficient set of each later stage time: 1..NTIME-1 in place, the step end in sE
        int tset[TB::NTIME + 1];
#pragma unroll
        for (int q = 1; q < TB::NTIME; ++q) tset[q] = q;
        tset[TB::NTIME] = sE;
        // coefficients at the later stage times (the last one, t + h, with τ-derivatives: it is the
        // next step's Jacobian set), and the factorisation for this h
        coef_eval(g, W, tset + 1, W.ctl + 4, TB::NTIME, 1u << (TB::NTIME - 1), false, cd, tab, M.nexpr, M.nx, mk);
        factorize(g, W, F, CJ, comps, M, k, h, s, TB::gam, scan);
        double b[NSL], Fv[NSL], Y[NSL], Ul[NSL];  // Ul: the last stage computed
        double U[kRolledStages<NW, ST> ? 1 : TB::S][NSL];  // the stages (unrolled loop)
        float isk[NSL];  // refinement stopping weights
#pragma unroll
        for (int sl = 0; sl < NSL; ++sl) isk[sl] = 1.0f / f64_to_f32(atol + rtol * fabs(y[sl]));
        if constexpr (kRolledStages<NW, ST>) {
          float c1 = 1e30f;
          int rk = A.refine;
          // the stage count read at run time: the compiler sees no fixed trip count to unroll or specialise
          const int nst = *reinterpret_cast<const volatile int*>(&kRos.nst);
#pragma unroll 1
          for (int st = 0; st < nst; ++st) {
            if (st == 0) {
#pragma unroll
              for (int sl = 0; sl < NSL; ++sl) b[sl] = f0[sl] + h * TB::d(0) * ft[sl];
            } else {
              // stage input: y + Σ A_st,j U_j, or the previous input plus U_{st-1}
              const bool inc = kRos.incr[st] != 0;
#pragma unroll
              for (int sl = 0; sl < NSL; ++sl) {
                const int i = comp_of<NW>(gt, sl);
                double v;
                if (inc) {
                  v = Y[sl] + Ul[sl];
                } else {
                  v = y[sl];
#pragma unroll 1
                  for (int j = 0; j < st; ++j) v += kRos.A[st][j] * W.Us[j][i];
                }
                Y[sl] = v;
                if (i < n) W.x[i] = v;
              }
              g.sync();
              const int q = kRos.tslot[st];
              matvec<NW, NSL>(g, W.x, W.cs[q < TB::NTIME ? q : sE], comps, M, k, Fv);
              const bool hd = kRos.hasd[st] != 0;
              const double hdst = h * kRos.d[st];
#pragma unroll
              for (int sl = 0; sl < NSL; ++sl) {
                const int i = comp_of<NW>(gt, sl);
                double cu = 0;
#pragma unroll 1
                for (int j = 0; j < st; ++j) cu += kRos.C[st][j] * W.Us[j][i];
                b[sl] = Fv[sl] + ih * cu;
                if (hd) b[sl] += hdst * ft[sl];
              }
            }
            // lazy refinement: the later stages share stage 1's W; they are refined only when stage
            // 1's first FP64 correction is at or above refine_skip (error-weight units)
            stage_solve(g, W, F, CJ, comps, M, k, s, rk, scan, isk, b, Ul, st == 0 ? &c1 : nullptr);
            if (st == 0) rk = (A.refine > 0 && c1 < A.refine_skip) ? 0 : A.refine;
#pragma unroll
            for (int sl = 0; sl < NSL; ++sl) W.Us[st][comp_of<NW>(gt, sl)] = Ul[sl];
          }
        } else {
#pragma unroll
        for (int sl = 0; sl < NSL; ++sl) b[sl] = f0[sl] + h * TB::d(0) * ft[sl];
        float c1 = 1e30f;
        stage_solve(g, W, F, CJ, comps, M, k, s, A.refine, scan, isk, b, U[0], &c1);
        // lazy refinement: the later stages share stage 1's W; they are refined only when stage 1's
        // first FP64 correction is at or above refine_skip (error-weight units)
        const int rk = (A.refine > 0 && c1 < A.refine_skip) ? 0 : A.refine;
#pragma unroll
        for (int st = 1; st < TB::S; ++st) {
          // stage input: y + Σ A_st,j U_j, or the previous input plus U_{st-1}
#pragma unroll
          for (int sl = 0; sl < NSL; ++sl) {
            const int i = comp_of<NW>(gt, sl);
            double v;
            if (TB::incremental(st)) {
              v = Y[sl] + U[st - 1][sl];
            } else {
              v = y[sl];
#pragma unroll
              for (int j = 0; j < st; ++j) if (TB::A(st, j) != 0.0) v += TB::A(st, j) * U[j][sl];
            }
            Y[sl] = v;
            if (i < n) W.x[i] = v;
          }
          g.sync();
          matvec<NW, NSL>(g, W.x, W.cs[tset[TB::tslot(st)]], comps, M, k, Fv);
#pragma unroll
          for (int sl = 0; sl < NSL; ++sl) {
            double cu = 0;
#pragma unroll
            for (int j = 0; j < st; ++j) cu += TB::C(st, j) * U[j][sl];
            b[sl] = Fv[sl] + ih * cu;
            if (TB::d(st) != 0.0) b[sl] += h * TB::d(st) * ft[sl];
          }
          stage_solve(g, W, F, CJ, comps, M, k, s, rk, scan, isk, b, U[st]);
        }
#pragma unroll
        for (int sl = 0; sl < NSL; ++sl) Ul[sl] = U[TB::S - 1][sl];
        }
        // new state (stiffly accurate: y1 = last stage input + last stage) and the FP64 error norm
        // of the last stage (the stage solutions are FP64 after refinement; only the
        // factorisation was FP32)
        double y1[NSL], err2;
        {
          double e2 = 0;
#pragma unroll
          for (int sl = 0; sl < NSL; ++sl) {
            const int i = comp_of<NW>(gt, sl);
            y1[sl] = Y[sl] + Ul[sl];
            if (i < n) {
              const double sk = atol + rtol * __longlong_as_double(max(dkey(fabs(y[sl])), dkey(fabs(y1[sl]))));
              const double q = Ul[sl] / sk;
              e2 += q * q;
            }
          }
          err2 = group_sum(g, W, e2) * inv_n;  // squared RMS error norm
        }
        // err2 >= 0: accepted when finite and at most 1, by its bit pattern (inf, NaN and any
        // sign-bit pattern compare above 1 as unsigned)
        if ((unsigned long long)dkey(err2) <= (unsigned long long)dkey(1.0)) {
          // accept: f(t1, y1) with the t1 coefficients, then dense output
#pragma unroll
          for (int sl = 0; sl < NSL; ++sl) { const int i = comp_of<NW>(gt, sl); if (i < n) W.x[i] = y1[sl]; }
          g.sync();
          if (g.wq == cw) {
            // PI controller fac = 0.9 err^-beta1 errold^beta2 (OrdinaryDiffEq's defaults for the
            // method's order), FP64 in both precisions; log(errold) is kept from the previous acceptance
            const double lerr = 0.5 * log(dmax(err2, 1e-20));
            double fac = 0.9 * exp(-TB::beta1 * lerr + TB::beta2 * lerrold);
            fac = dmin(10.0, dmax(0.2, fac));
            if (rejected) fac = dmin(fac, 1.0);
            lerrold = dmax(lerr, kLogErrFloor);
            publish(h * fac, tn);
          }
          // f(t1, y1) and the next step's ∂f/∂τ = (dJ/dτ)(t1) y1, both from the t1 coefficient set,
          // which becomes the next step's Jacobian set
          double f1[NSL];
          matvec_jd<NW, NSL>(g, W.x, W.cs[sE], comps, M, k, f1, ft);
          { const int tsw = sJ; sJ = sE; sE = tsw; }
          if (taus && jout < A.ntau && dkey(taus[jout]) <= dkey(tn)) {
            // continuous extension y(t + θh) = (1-θ) y + θ (y1 + (1-θ)(K0 + θ K1 + θ² K2))
            double K[TB::NDENSE][NSL];
#pragma unroll
            for (int r = 0; r < TB::NDENSE; ++r)
#pragma unroll
              for (int sl = 0; sl < NSL; ++sl) {
                double v = 0;
#pragma unroll
                for (int j = 0; j < TB::S; ++j) {
                  if (TB::dense(r, j) == 0.0) continue;
                  double uj;
                  if constexpr (kRolledStages<NW, ST>) uj = W.Us[j][comp_of<NW>(gt, sl)];
                  else uj = U[j][sl];
                  v += TB::dense(r, j) * uj;
                }
                K[r][sl] = v;
              }
            g.sync();  // x readers of the f1 product are done
            while (jout < A.ntau && dkey(taus[jout]) <= dkey(tn)) {
              const double tau = taus[jout];
              const double th = (tau - t) / (tn - t), th1 = 1.0 - th;
              double yo[NSL];
#pragma unroll
              for (int sl = 0; sl < NSL; ++sl) yo[sl] = th1 * y[sl] + th * (y1[sl] + th1 * (K[0][sl] + th * (K[1][sl] + th * K[2][sl])));
              emit_output(g, W, A, cd, tab, comps, M, mk, tau, yo, item, jout);
              ++jout;
            }
          }
          t = tn;
#pragma unroll
          for (int sl = 0; sl < NSL; ++sl) { y[sl] = y1[sl]; f0[sl] = f1[sl]; }
          ++nacc;
          rejected = false; nonfinite = false;
        } else {
          ++nrej;
          rejected = true;
          if ((dkey(err2) & 0x7ff0000000000000ll) == 0x7ff0000000000000ll) nonfinite = true;  // inf or NaN
          if (g.wq == cw) publish(nonfinite ? 0.2 * h : h * dmax(0.2, 0.9 * exp(-0.5 * TB::rej * log(err2))), t);
          // J's coefficients (at t) and ∂f/∂τ stay valid; only the factorisation changes
        }
      }
    }
    // saved times never reached (failed mode): zero
    if (taus) {
      for (; jout < A.ntau; ++jout) {
        if (A.output == SBZ_OUT_SOURCES && gt < 3) A.out[((size_t)item * A.ntau + jout) * 3 + gt] = 0;
        if (A.output == SBZ_OUT_SOURCES4 && gt < 4) A.out[((size_t)item * A.ntau + jout) * 4 + gt] = 0;
        if (A.output == SBZ_OUT_FACTORS && gt < 7) A.out[((size_t)item * A.ntau + jout) * 7 + gt] = 0;
        if (A.output == SBZ_OUT_STATE) for (int i = gt; i < n; i += NT) A.out[((size_t)item * A.ntau + jout) * n + i] = 0;
      }
    }
    bool finite = true;
#pragma unroll
    for (int sl = 0; sl < NSL; ++sl) { const int i = comp_of<NW>(gt, sl); if (i < n && !isfinite(y[sl])) finite = false; }
    finite = group_sum(g, W, finite ? 0.0 : 1.0) == 0.0;
    if (status == SBZ_OK && !finite) status = SBZ_NONFINITE;
    if (A.output == SBZ_OUT_DELTA_M) {
      // Δ_m(τ0) = Σ ρ_s Δ_s / Σ ρ_s over c, b, massive ν   (src/observables/fourier.jl:39-52)
      const int so = kNSets - 1;
      g.sync();
      coef_eval(g, W, &so, &tend, 1, 0u, false, cd, tab, M.nexpr, M.nx, mk);
#pragma unroll
      for (int sl = 0; sl < NSL; ++sl) { const int i = comp_of<NW>(gt, sl); if (i < n) W.x[i] = y[sl]; }
      g.sync();
      if (g.wq == 0) {
        double I0 = 0, I1 = 0, Ir = 0;
        if (g.lane < M.nx) {
          const int base = M.oH + g.lane * (M.Lh + 1);
          I0 = cd->Wq[g.lane] * W.B[0][B_E + g.lane] * W.x[base];
          I1 = cd->Wq[g.lane] * cd->xq[g.lane] * W.x[base + 1];
          Ir = cd->Wq[g.lane] * W.B[0][B_E + g.lane];
        }
        I0 = warp_sum(I0); I1 = warp_sum(I1); Ir = warp_sum(Ir);
        if (gt == 0) {
          const double ia = W.B[0][B_IA], Hc = W.B[0][B_H];
          double num = cd->Oc0 * (W.x[1] + 3 * Hc * W.x[2] * mk.ik2) + cd->Ob0 * (W.x[3] + 3 * Hc * W.x[4] * mk.ik2);
          double den = cd->Oc0 + cd->Ob0;
          num += cd->wh * ia * (I0 + 3 * Hc * I1 * mk.ik);
          den += cd->wh * ia * Ir;
          A.out[item] = num / den;
        }
      }
    }
    if (gt == 0) {
      if (A.status) A.status[item] = status;
      if (A.steps) { A.steps[2 * item] = nacc; A.steps[2 * item + 1] = nrej; }
    }
    g.sync();
  }
}

// Register budget: four-warp groups run at most two per SM (tail-bound spectra), so they may use up
// to 256 registers per thread and need not spill; eight-warp groups (one 256-thread block per SM:
// one mode per SM, two warps per sub-partition) likewise; narrower groups keep three 128-thread
// blocks per SM (throughput-bound batches), accepting a few spilled registers for the occupancy.
template <int NW, int NSL, typename ST>
__global__ void __launch_bounds__(NW >= 8 ? 256 : 128, NW >= 8 ? 1 : NW >= 4 ? 2 : 3) pt_kernel(PtArgs A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ModelDesc& M = *reinterpret_cast<ModelDesc*>(smem_raw);
  CompDesc* comps = reinterpret_cast<CompDesc*>(smem_raw + ((sizeof(ModelDesc) + 15) & ~size_t(15)));
  const size_t comp_bytes = ((size_t)A.model_n * sizeof(CompDesc) + 15) & ~size_t(15);
  using Mem = ModeMem<NW, NSL, ST>;
  Mem* Wm = reinterpret_cast<Mem*>(smem_raw + ((sizeof(ModelDesc) + 15) & ~size_t(15)) + comp_bytes);
  // block-wide copy of the model descriptors
  for (int i = threadIdx.x; i < (int)sizeof(ModelDesc) / 4; i += blockDim.x) reinterpret_cast<int*>(&M)[i] = reinterpret_cast<const int*>(A.model)[i];
  for (int i = threadIdx.x; i < A.model_n * (int)sizeof(CompDesc) / 4; i += blockDim.x) reinterpret_cast<int*>(comps)[i] = reinterpret_cast<const int*>(A.comps)[i];
  __syncthreads();
  const int grp = threadIdx.x / (32 * NW);
  Grp<NW> g;
  g.gt = threadIdx.x - grp * 32 * NW;
  g.lane = threadIdx.x & 31;
  g.wq = g.gt >> 5;
  g.bar = 1 + grp;
  g.rp = 0;
  init_lane_consts<NW, NSL>(g, M, comps);
  pt_body<NW, NSL, ST>(A, M, comps, Wm[grp], g);
}

template <int NW, int NSL, typename ST>
int launch_nw(const PtArgs& A, int warps_per_block, int blocks_per_sm, int num_sms, cudaStream_t stream) {
  using Mem = ModeMem<NW, NSL, ST>;
  const int wpb = warps_per_block < NW ? NW : warps_per_block > 4 ? 4 : warps_per_block;  // ≤ 128 threads, or one 8-warp group
  const int groups = wpb / NW;
  const size_t head = ((sizeof(ModelDesc) + 15) & ~size_t(15)) + (((size_t)A.model_n * sizeof(CompDesc) + 15) & ~size_t(15));
  const size_t smem = head + groups * sizeof(Mem);
  auto kern = pt_kernel<NW, NSL, ST>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return SBZ_ERR_CUDA;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * NW * groups, smem) != cudaSuccess) return SBZ_ERR_CUDA;
  per_sm = per_sm < 1 ? 1 : per_sm;
  if (blocks_per_sm > 0 && blocks_per_sm < per_sm) per_sm = blocks_per_sm;
  const int want = (A.nitems + groups - 1) / groups;
  const int grid = want < num_sms * per_sm ? want : num_sms * per_sm;
  kern<<<grid > 0 ? grid : 1, 32 * NW * groups, smem, stream>>>(A);
  return cudaGetLastError() == cudaSuccess ? SBZ_OK : SBZ_ERR_CUDA;
}

// f = J(τ) y and ∂f/∂τ = (dJ/dτ) y for single modes (one warp each): the model's right-hand side
// as the integrator evaluates it.
template <int NSL>
__global__ void __launch_bounds__(32) rhs_kernel(PtArgs A, const double* __restrict__ y_in, const double* __restrict__ tau_in,
                                                 double* __restrict__ f_out, double* __restrict__ ft_out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ModelDesc& M = *reinterpret_cast<ModelDesc*>(smem_raw);
  CompDesc* comps = reinterpret_cast<CompDesc*>(smem_raw + ((sizeof(ModelDesc) + 15) & ~size_t(15)));
  const size_t comp_bytes = ((size_t)A.model_n * sizeof(CompDesc) + 15) & ~size_t(15);
  using Mem = ModeMem<1, NSL, double>;
  Mem& W = *reinterpret_cast<Mem*>(smem_raw + ((sizeof(ModelDesc) + 15) & ~size_t(15)) + comp_bytes);
  Grp<1> g;
  g.gt = threadIdx.x & 31; g.lane = g.gt; g.wq = 0; g.bar = 0; g.rp = 0;
  for (int i = g.gt; i < (int)sizeof(ModelDesc) / 4; i += 32) reinterpret_cast<int*>(&M)[i] = reinterpret_cast<const int*>(A.model)[i];
  for (int i = g.gt; i < A.model_n * (int)sizeof(CompDesc) / 4; i += 32) reinterpret_cast<int*>(comps)[i] = reinterpret_cast<const int*>(A.comps)[i];
  __syncwarp();
  init_lane_consts<1, NSL>(g, M, comps);
  const int n = M.n, item = blockIdx.x;
  for (int i = g.gt; i < kNSets * (int)(sizeof(CSet) / sizeof(double)); i += 32) reinterpret_cast<double*>(W.cs)[i] = 0;
  for (int i = n + g.gt; i <= 32 * NSL; i += 32) W.x[i] = 0;
  __syncwarp();
  const int c = A.item_cosmo ? A.item_cosmo[item] : 0;
  const CosmoDesc* cd = A.cosmos + c;
  const double* tab = A.tables + (size_t)c * A.table_stride;
  ModeK mk;
  mk.k = A.item_k[item]; mk.k2 = mk.k * mk.k; mk.ik = 1.0 / mk.k; mk.ik2 = mk.ik * mk.ik;
  const double tau = tau_in[item];
  const int so = 0;
  coef_eval(g, W, &so, &tau, 1, 1u, false, cd, tab, M.nexpr, M.nx, mk);
  for (int i = g.gt; i < n; i += 32) W.x[i] = y_in[(size_t)item * n + i];
  __syncwarp();
  double f[NSL], ft[NSL];
  matvec<1, NSL>(g, W.x, W.cs[0], comps, M, mk.k, f);
  matvec_dtau<1, NSL>(g, W.x, W.cs[0], comps, M, mk.k, ft);
#pragma unroll
  for (int sl = 0; sl < NSL; ++sl) {
    const int i = g.gt + 32 * sl;
    if (i < n) { f_out[(size_t)item * n + i] = f[sl]; ft_out[(size_t)item * n + i] = ft[sl]; }
  }
}

template <int NSL>
int rhs_launch_ns(const PtArgs& A, const double* y, const double* tau, double* f, double* ft, cudaStream_t st) {
  const size_t smem = ((sizeof(ModelDesc) + 15) & ~size_t(15)) + (((size_t)A.model_n * sizeof(CompDesc) + 15) & ~size_t(15)) +
                      sizeof(ModeMem<1, NSL, double>);
  auto kern = rhs_kernel<NSL>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return SBZ_ERR_CUDA;
  kern<<<A.nitems, 32, smem, st>>>(A, y, tau, f, ft);
  return cudaGetLastError() == cudaSuccess ? SBZ_OK : SBZ_ERR_CUDA;
}

}  // namespace ptk
}  // namespace sbz
