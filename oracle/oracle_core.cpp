// CPU oracle, core physics and integrator.  TEST INFRASTRUCTURE ONLY (see oracle.h).
//
// Restates, in FP64 C++, the reference's equations:
//   constants            src/constants.jl:3-50
//   metric / GR          src/models/metric.jl:6-28, src/models/gravity.jl:6-45 (pt eqs :37-42)
//   constant-w species   src/models/generic_species.jl:6-60
//   baryons + RECFAST    src/models/baryons.jl:14-212
//   photons              src/models/photons.jl:6-73
//   neutrinos            src/models/neutrinos.jl:6-143 (momentum quadrature :55-60)
//   CDM, Lambda          src/models/dark_matter.jl:6-9, src/models/dark_energy.jl:6-17
//   inflation            src/models/inflation.jl:1-14
//   LCDM couplings/ICs   src/models/cosmologies.jl:27-114, 221-227
//   background solve     src/solve.jl:158-203 (a=1 callback), 427-435
//   background spline    src/utils.jl:118-127 (cubic Hermite spline of the bg unknowns)
//   perturbation solve   src/solve.jl:496-569
// The integrator is a Rosenbrock method in transformed form: Rodas5P (Steinebach 2023, order
// 5(4)), the reference's default (src/solve.jl:320,339; OrdinaryDiffEqRosenbrock, not vendored,
// restated from the published tableau), or the Hairer-Wanner RODAS (order 4(3)).  Parity with
// the reference is at the level of outputs, not steps.  Linear systems are solved with dense
// LU and partial pivoting (the reference uses KLU on the same matrix).
#include "oracle.h"
#include "jet.hpp"
#include <vector>
#include <cstdint>
#include <algorithm>
#include <cstring>
#include <cstdio>
#include <cmath>
#include <limits>
#include <type_traits>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

// ------------------------------------------------------------------------------------------
// constants (CODATA 2018, IAU parsec, PeriodicTable atomic masses) - src/constants.jl
namespace K {
const double PI = 3.14159265358979323846;
const double c = 299792458.0;
const double hP = 6.62607015e-34;
const double hbar = hP / (2 * PI);
const double kB = 1.380649e-23;
const double GN = 6.67430e-11;
const double sigmaSB = 5.670374419e-8;
const double aR = 4.0 / c * sigmaSB;
const double sigmaT = 6.6524587321e-29;
const double me = 9.1093837015e-31;
const double amu = 1.66053906660e-27;
const double mH = 1.008 * amu;
const double mHe = 4.0026022 * amu;
const double pc = 3.0856775814913673e16;
const double Mpc = 1e6 * pc;
const double H100 = 100.0 * 1000.0 / Mpc;
const double eV = 1.602176634e-19;
// transitions: E = h * (c / lambda)
inline double E(double lam) { return hP * (c / lam); }
const double lamH2s1s = 121.56700e-9;
const double EHinf1s = E(91.17534e-9), EH2s1s = E(lamH2s1s), EHinf2s = EHinf1s - EH2s1s;
const double lamHe2p1s = 58.43344e-9;
const double EHeinf1s = E(50.42590e-9), EHe2s1s = E(60.14045e-9), EHe2p1s = E(lamHe2p1s);
const double EHe2p2s = EHe2p1s - EHe2s1s, EHeinf2s = EHeinf1s - EHe2s1s;
const double EHepinf1s = 54.4178 * eV;
const double lamHet2p1s = 59.1411e-9;
const double EHetinf2s = E(260.0463e-9), EHet2p1s = E(lamHet2p1s), EHet2s1s = E(62.5563e-9);
const double EHet2p2s = EHet2p1s - EHet2s1s;
const double fHe2p1s = c / lamHe2p1s, fHet2p1s = c / lamHet2p1s;
}  // namespace K

// ------------------------------------------------------------------------------------------
// momentum quadrature (src/models/neutrinos.jl:55-60): N-point Gauss rule for the measure
// x^2 f0(x) dx, f0 = 1/(e^x+1), after the substitution u = 1/(1+x/100) (x = 100(1-u)/u).
// Built here by the discretised Stieltjes procedure + Golub-Welsch on the Jacobi matrix.
static void jacobi_eig(int n, double* A, double* V) {  // symmetric, A overwritten by diag
  for (int i = 0; i < n; ++i) for (int j = 0; j < n; ++j) V[i * n + j] = (i == j);
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0; for (int i = 0; i < n; ++i) for (int j = i + 1; j < n; ++j) off += A[i * n + j] * A[i * n + j];
    if (off < 1e-30) break;
    for (int p = 0; p < n; ++p) for (int q = p + 1; q < n; ++q) {
      double apq = A[p * n + q]; if (std::fabs(apq) < 1e-300) continue;
      double theta = (A[q * n + q] - A[p * n + p]) / (2 * apq);
      double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1));
      double cs = 1 / std::sqrt(t * t + 1), sn = t * cs;
      for (int k = 0; k < n; ++k) { double akp = A[k * n + p], akq = A[k * n + q]; A[k * n + p] = cs * akp - sn * akq; A[k * n + q] = sn * akp + cs * akq; }
      for (int k = 0; k < n; ++k) { double apk = A[p * n + k], aqk = A[q * n + k]; A[p * n + k] = cs * apk - sn * aqk; A[q * n + k] = sn * apk + cs * aqk; }
      for (int k = 0; k < n; ++k) { double vkp = V[k * n + p], vkq = V[k * n + q]; V[k * n + p] = cs * vkp - sn * vkq; V[k * n + q] = sn * vkp + cs * vkq; }
    }
  }
}

static int momentum_quadrature(int N, double* xs, double* Ws) {
  if (N < 1 || N > 16) return -1;
  // discretised measure: composite 20-point Gauss-Legendre on 400 panels of (0,1)
  const int npan = 400, ng = 20;
  double gx[ng], gw[ng];
  for (int i = 0; i < ng; ++i) {  // Legendre nodes by Newton
    double z = std::cos(K::PI * (i + 0.75) / (ng + 0.5)), pp = 0;
    for (int it = 0; it < 100; ++it) {
      double p1 = 1, p2 = 0;
      for (int j = 1; j <= ng; ++j) { double p3 = p2; p2 = p1; p1 = ((2 * j - 1) * z * p2 - (j - 1) * p3) / j; }
      pp = ng * (z * p1 - p2) / (z * z - 1);
      double z1 = z; z = z1 - p1 / pp; if (std::fabs(z - z1) < 1e-16) break;
    }
    gx[i] = z; gw[i] = 2 / ((1 - z * z) * pp * pp);
  }
  std::vector<double> u, w;
  for (int p = 0; p < npan; ++p) {
    double a = double(p) / npan, b = double(p + 1) / npan;
    for (int i = 0; i < ng; ++i) {
      double uu = 0.5 * (a + b) + 0.5 * (b - a) * gx[i];
      double x = 100 * (1 - uu) / uu;
      double dens = (100.0 / (uu * uu)) * x * x / (std::exp(x) + 1);
      u.push_back(uu); w.push_back(0.5 * (b - a) * gw[i] * dens);
    }
  }
  const size_t M = u.size();
  std::vector<double> pprev(M, 0.0), pcur(M, 1.0), pnext(M);
  double al[16], be[16], nrm_prev = 1;
  for (int k = 0; k < N; ++k) {
    double nrm = 0, mom = 0;
    for (size_t i = 0; i < M; ++i) { nrm += w[i] * pcur[i] * pcur[i]; mom += w[i] * u[i] * pcur[i] * pcur[i]; }
    al[k] = mom / nrm; be[k] = (k == 0) ? nrm : nrm / nrm_prev; nrm_prev = nrm;
    for (size_t i = 0; i < M; ++i) pnext[i] = (u[i] - al[k]) * pcur[i] - (k ? be[k] : 0.0) * pprev[i];
    pprev.swap(pcur); pcur.swap(pnext);
  }
  double A[256], V[256];
  for (int i = 0; i < N * N; ++i) A[i] = 0;
  for (int i = 0; i < N; ++i) { A[i * N + i] = al[i]; if (i + 1 < N) A[i * N + i + 1] = A[(i + 1) * N + i] = std::sqrt(be[i + 1]); }
  jacobi_eig(N, A, V);
  std::vector<std::pair<double, double>> xw;
  for (int i = 0; i < N; ++i) {
    double uu = A[i * N + i];
    xw.push_back({100 * (1 - uu) / uu, be[0] * V[0 * N + i] * V[0 * N + i]});
  }
  std::sort(xw.begin(), xw.end());
  for (int i = 0; i < N; ++i) { xs[i] = xw[i].first; Ws[i] = xw[i].second; }
  return 0;
}

// ------------------------------------------------------------------------------------------
// cosmology: parameters and derived constants
struct Cosmo {
  double h, Oc0, Ob0, T0, Neff, YHe, As, ns, m_eV, Nnu;
  int Lg, Ln, Lh, nx, Hswitch, Heswitch, reion;
  double H0si, Og0, On0, Oh0, OL0, fHe, kpivot, Th0, y0, Irho0;
  double xq[16], Wq[16], dlnf[16];
  double rtol_bg, atol_bg, rtol_pt, atol_pt, tau_ini, tau_max;
  long maxiters;
  int alg_bg, alg_pt, pt_linsolve;
};

static void cosmo_init(Cosmo& P, const orc_params* p, const orc_model* m, const orc_opts* o) {
  using namespace K;
  P.h = p->h; P.Oc0 = p->Omega_c; P.Ob0 = p->Omega_b; P.T0 = p->T0; P.Neff = p->Neff; P.YHe = p->YHe;
  P.As = std::exp(p->ln_As1e10) / 1e10; P.ns = p->ns; P.m_eV = p->m_nu_eV; P.Nnu = p->N_nu;
  P.Lg = m->lmax_g; P.Ln = m->lmax_nu; P.Lh = m->lmax_h; P.nx = m->nx;
  P.Hswitch = m->Hswitch; P.Heswitch = m->Heswitch; P.reion = m->reionization;
  P.H0si = H100 * P.h;
  // photons: src/models/photons.jl:45
  P.Og0 = PI * PI / 15 * std::pow(kB * P.T0, 4) / (std::pow(hbar, 3) * std::pow(c, 5)) * 8 * PI * GN / (3 * P.H0si * P.H0si);
  // massless nu: src/models/cosmologies.jl:78-81
  P.On0 = P.Neff * 7.0 / 8.0 * std::pow(4.0 / 11.0, 4.0 / 3.0) * P.Og0;
  // massive nu: src/models/neutrinos.jl:78-86
  P.Oh0 = 0; P.Th0 = std::pow(4.0 / 11.0, 1.0 / 3.0) * P.T0; P.y0 = 0; P.Irho0 = 0;
  if (P.nx > 0) {
    momentum_quadrature(P.nx, P.xq, P.Wq);
    double mkg = P.m_eV * eV / (c * c);
    P.y0 = mkg * c * c / (kB * P.Th0);
    for (int i = 0; i < P.nx; ++i) {
      P.Irho0 += P.Wq[i] * std::sqrt(P.xq[i] * P.xq[i] + P.y0 * P.y0);
      P.dlnf[i] = -P.xq[i] / (1 + std::exp(-P.xq[i]));
    }
    P.Oh0 = P.Nnu * 8 * PI / 3 * 2 / (2 * PI * PI) * std::pow(kB * P.Th0, 4) / std::pow(hbar * c, 3) * P.Irho0 / (std::pow(P.H0si * c, 2) / GN);
  }
  // closure on the last species (Lambda): src/models/cosmologies.jl:221-227
  P.OL0 = 1 - (P.Og0 + P.On0 + P.Oc0 + P.Ob0 + P.Oh0);
  // src/models/baryons.jl:151, src/models/inflation.jl:6
  P.fHe = P.YHe / (mHe / mH * (1 - P.YHe));
  P.kpivot = 0.05 / Mpc / (H100 / c) / P.h;
  P.rtol_bg = o->bg_rtol; P.atol_bg = o->bg_atol; P.rtol_pt = o->pt_rtol; P.atol_pt = o->pt_atol;
  P.tau_ini = o->tau_ini; P.tau_max = o->tau_max; P.maxiters = o->maxiters;
  P.alg_bg = o->alg_bg; P.alg_pt = o->alg_pt; P.pt_linsolve = o->pt_linsolve;
}

template <class S> inline S smoothifelse(const S& x, const S& v1, const S& v2, double k) {
  return 0.5 * ((v1 + v2) + (v2 - v1) * tanh(k * x));  // src/utils.jl:37
}

template <class S> struct BgOut { S a, ap, Hc, kd, Xe, Tb, DT, cs2, XHepp, Om; };

// Background right-hand side.  y = [a, _kappa, dT(=Tb-Tgamma), XH+, XHe+].
template <class S>
static void bg_rhs(const Cosmo& P, const S* y, S* dy, BgOut<S>* out) {
  using namespace K;
  const S a = y[0];
  const S ia = 1.0 / a, ia3 = ia * ia * ia, ia4 = ia3 * ia;
  S Om = (P.Og0 + P.On0) * ia4 + (P.Oc0 + P.Ob0) * ia3 + S(P.OL0);
  if (P.nx > 0) {
    S Ir(0.0);
    for (int i = 0; i < P.nx; ++i) Ir += P.Wq[i] * sqrt(P.xq[i] * P.xq[i] + (P.y0 * P.y0) * (a * a));
    Om += (P.Oh0 / P.Irho0) * Ir * ia4;
  }
  const S ap = sqrt(Om) * a * a;  // src/models/gravity.jl:31
  const S Hc = ap * ia;
  const S Hsi = P.H0si * Hc * ia;
  const S Tg = P.T0 * ia;
  const S dT = y[2];
  const S Tb = dT + Tg;
  const S XH = y[3], XHe = y[4];
  const S nH = (1 - P.YHe) * (3 / (8 * PI)) * P.Ob0 * ia3 * (P.H0si * P.H0si / GN) / mH;
  const S nHe = P.fHe * nH;
  const S beta = 1.0 / (kB * Tb);
  const S lam = hP / sqrt((2 * PI * me * kB) * Tb);
  const S lam3 = lam * lam * lam;
  // He++ Saha (src/models/baryons.jl:68-69)
  const S RHep = exp(-beta * EHepinf1s) / (nH * lam3);
  const S den = 1 + P.fHe + RHep;
  const S XHepp = 2 * RHep * P.fHe / den / (1 + sqrt(1 + 4 * RHep * P.fHe / (den * den)));
  S Xe = XH + P.fHe * XHe + XHepp;
  if (P.reion) {  // src/models/baryons.jl:128-138,201-205
    const S opz = ia;  // 1+z
    {
      double zr = 7.6711, dz = 0.5, n = 1.5, Xm = 1 + P.fHe;
      double kk = 1 / (n * std::pow(1 + zr, n - 1) * dz);
      Xe += smoothifelse(std::pow(1 + zr, n) - pow(opz, n), S(0.0), S(Xm), kk);
    }
    {
      double zr = 3.5, dz = 0.5, Xm = P.fHe;
      double kk = 1 / (1.0 * dz);
      Xe += smoothifelse((1 + zr) - opz, S(0.0), S(Xm), kk);
    }
  }
  const S ne = Xe * nH;
  const S conv = a / P.H0si;
  const S kd = -conv * ne * sigmaT * c;  // src/models/baryons.jl:176
  const S Tg4 = Tg * Tg * Tg * Tg;
  const S DT = -2 * Tb * Hc - conv * (8.0 / 3.0) * sigmaT * aR * Tg4 / (me * c) * Xe / (1 + P.fHe + Xe) * dT;
  dy[0] = ap;
  dy[1] = kd;
  dy[2] = DT + Tg * Hc;  // D(dT) = DT - D(Tgamma), D(Tgamma) = -Tgamma*H
  // hydrogen (src/models/baryons.jl:41-54,75-84)
  const double FH = (P.Hswitch == 0) ? 1.14 : 1.125;
  const S TT = Tb / 1e4;
  const S alH = FH * 1e-19 * 4.309 * pow(TT, -0.6166) / (1 + 0.6703 * pow(TT, 0.5300));
  const S beH = alH / lam3 * exp(-beta * EHinf2s);
  S KHfit(1.0);
  if (P.Hswitch == 1) {
    const S la = log(a);
    const S g1 = (la + 7.28) / 0.18, g2 = (la + 6.73) / 0.33;
    KHfit = 1 + (-0.14) * exp(-(g1 * g1)) + 0.079 * exp(-(g2 * g2));
  }
  const double LH = 8.2245809, LHe = 51.3;
  const S KH = KHfit / (8 * PI) * (lamH2s1s * lamH2s1s * lamH2s1s) / Hsi;
  const S CHraw = (1 + KH * LH * nH * (1 - XH)) / (1 + KH * (LH + beH) * nH * (1 - XH));
  const S CH = smoothifelse(XH - 0.99, CHraw, S(1.0), 1e3);
  dy[3] = -conv * CH * (alH * XH * ne - beH * (1 - XH) * exp(-beta * EH2s1s));
  // helium singlet (src/models/baryons.jl:42,57-65,88-110)
  auto alHefit = [&](double q, double p) {
    const double T1 = std::pow(10.0, 5.114), T2 = 3.0;
    const S s2 = sqrt(Tb / T2), s1 = sqrt(Tb / T1);
    return q / (s2 * pow(1 + s2, 1 - p) * pow(1 + s1, 1 + p));
  };
  const S alHe = alHefit(std::pow(10.0, -16.744), 0.711);
  const S beHe = 4 * alHe / lam3 * exp(-beta * EHeinf2s);
  const S invK0 = 8 * PI * Hsi / (K::lamHe2p1s * K::lamHe2p1s * K::lamHe2p1s);
  const double eps = 1e-9;
  S invK1(0.0), invK2(0.0), dXHet(0.0);
  if (P.Heswitch == 6) {
    const double A2ps = 1.798287e9, A2pt = 177.58;
    auto gamHe = [&](double A, double sig, double f) {
      return 3 * A * P.fHe * (1 - XHe + eps) * (c * c) /
             (8 * PI * sig * sqrt(2 * PI / (beta * mHe * c * c)) * (1 - XH + eps) * (f * f * f));
    };
    const S tauHe = 3 * A2ps * nHe * (1 - XHe + eps) / invK0;
    invK1 = -exp(-tauHe) * invK0;
    const S g2ps = gamHe(A2ps, 1.436289e-22, fHe2p1s);
    invK2 = A2ps / (1 + 0.36 * pow(g2ps, 0.86)) * 3 * nHe * (1 - XHe);
    const S alHet = alHefit(std::pow(10.0, -16.306), 0.761);
    const S beHet = 4.0 / 3.0 * alHet / lam3 * exp(-beta * EHetinf2s);
    const S tauHet = A2pt * nHe * (1 - XHe + eps) * 3 * (K::lamHet2p1s * K::lamHet2p1s * K::lamHet2p1s) / (8 * PI * Hsi);
    const S pHet = (1 - exp(-tauHet)) / tauHet;
    const S g2pt = gamHe(A2pt, 1.484872e-22, fHet2p1s);
    const S CHetnum = A2pt * (pHet + 1 / (1 + 0.66 * pow(g2pt, 0.9)) / 3) * exp(-beta * EHet2p2s);
    const S CHet = (eps + CHetnum) / (eps + CHetnum + beHet);
    dXHet = -conv * CHet * (alHet * XHe * ne - beHet * (1 - XHe) * 3 * exp(-beta * EHet2s1s));
  }
  const S KHe = 1 / (invK0 + invK1 + invK2);
  const S e22 = exp(-beta * EHe2p2s);
  const S CHeraw = (e22 + KHe * LHe * nHe * (1 - XHe)) / (e22 + KHe * (LHe + beHe) * nHe * (1 - XHe));
  const S CHe = smoothifelse(XHe - 0.99, CHeraw, S(1.0), 1e3);
  const S dXHes = -conv * CHe * (alHe * XHe * ne - beHe * (1 - XHe) * exp(-beta * EHe2s1s));
  dy[4] = dXHes + dXHet;
  if (out) {
    out->a = a; out->ap = ap; out->Hc = Hc; out->kd = kd; out->Xe = Xe; out->Tb = Tb; out->DT = DT;
    out->XHepp = XHepp; out->Om = Om;
    const S muc2 = mH * c * c / (1 + (mH / mHe - 1) * P.YHe + Xe * (1 - P.YHe));
    out->cs2 = kB / muc2 * (Tb - DT / (3 * Hc));  // src/models/baryons.jl:182-183
  }
}

// ------------------------------------------------------------------------------------------
// Rosenbrock tableaus in the transformed (W = 1/(h gamma) I - J) form of Hairer & Wanner,
// Solving ODEs II, IV.7 (eq. 7.25):
//   W U_i = f(t + c_i h, y + sum_j A_ij U_j) + sum_j (C_ij / h) U_j + h d_i f_t,
//   y1 = y + sum_j m_j U_j,  error estimate = U_s (the last stage; the embedded solution omits it).
// Step-size control is the PI controller fac = 0.9 err^-beta1 errold^beta2 (clamped to [0.2, 10]),
// with rejections scaled by max(0.2, 0.9 err^-rej).
// Dense output (ndense = 3): y(t + θh) = (1-θ) y + θ (y1 + (1-θ)(K0 + θ K1 + θ² K2)) with
// K_r = sum_j H_rj U_j; ndense = 0: cubic Hermite through (y, f) at both ends.
struct Tableau {
  int s;
  double c[8], d[8], A[8][8], C[8][8], m[8];
  double beta1, beta2, rej;
  int ndense;
  double H[3][8];
};

// RODAS (Hairer & Wanner, order 4(3), stiffly accurate): 6 stages.
static Tableau make_rodas4() {
  Tableau T{};
  T.s = 6;
  const double c2 = 0.386, c3 = 0.21, c4 = 0.63;
  const double a21 = 1.544;
  const double a31 = 0.9466785280815826, a32 = 0.2557011698983284;
  const double a41 = 3.314825187068521, a42 = 2.896124015972201, a43 = 0.9986419139977817;
  const double a51 = 1.221224509226641, a52 = 6.019134481288629, a53 = 12.53708332932087, a54 = -0.6878860361058950;
  const double Cs[6][6] = {{0}, {-5.6688}, {-2.430093356833875, -0.2063599157091915},
                           {-0.1073529058151375, -9.594562251023355, -20.47028614809616},
                           {7.496443313967647, -10.24680431464352, -33.99990352819905, 11.70890893206160},
                           {8.083246795921522, -7.981132988064893, -31.52159432874371, 16.31930543123136, -6.058818238834054}};
  const double cs[6] = {0, c2, c3, c4, 1, 1}, ds[6] = {0.25, -0.1043, 0.1035, -0.0362, 0, 0};
  for (int i = 0; i < 6; ++i) { T.c[i] = cs[i]; T.d[i] = ds[i]; for (int j = 0; j < i; ++j) T.C[i][j] = Cs[i][j]; }
  T.A[1][0] = a21; T.A[2][0] = a31; T.A[2][1] = a32; T.A[3][0] = a41; T.A[3][1] = a42; T.A[3][2] = a43;
  const double a5[4] = {a51, a52, a53, a54};
  for (int j = 0; j < 4; ++j) { T.A[4][j] = a5[j]; T.A[5][j] = a5[j]; T.m[j] = a5[j]; }
  T.A[5][4] = 1; T.m[4] = 1; T.m[5] = 1;
  T.beta1 = 0.175; T.beta2 = 0.1; T.rej = 0.25;
  return T;
}

// Rodas5P (Steinebach 2023, order 5(4), stiffly accurate; the reference's default integrator,
// src/solve.jl:320,339): 8 stages; stages 6-8 at t + h, each adding one correction.  The PI
// exponents are OrdinaryDiffEq's defaults for an order-5 method (7/50, 2/25), rejections by
// 0.9 err^-7/50.
static Tableau make_rodas5p() {
  Tableau T{};
  T.s = 8;
  const double gam = 0.21193756319429014;
  const double cs[8] = {0, 0.6358126895828704, 0.4095798393397535, 0.9769306725060716, 0.4288403609558664, 1, 1, 1};
  const double ds[8] = {gam, -0.42387512638858027, -0.3384627126235924, 1.8046452872882734, 2.325825639765069, 0, 0, 0};
  const double As[6][5] = {{0},
                           {3.0},
                           {2.849394379747939, 0.45842242204463923},
                           {-6.954028509809101, 2.489845061869568, -10.358996098473584},
                           {2.8029986275628964, 0.5072464736228206, -0.3988312541770524, -0.04721187230404641},
                           {-7.502846399306121, 2.561846144803919, -11.627539656261098, -0.18268767659942256, 0.030198172008377946}};
  const double Cs[8][7] = {{0},
                           {-14.155112264123755},
                           {-17.97296035885952, -2.859693295451294},
                           {147.12150275711716, -1.41221402718213, 71.68940251302358},
                           {165.43517024871676, -0.4592823456491126, 42.90938336958603, -5.961986721573306},
                           {24.854864614690072, -3.0009227002832186, 47.4931110020768, 5.5814197821558125, -0.6610691825249471},
                           {30.91273214028599, -3.1208243349937974, 77.79954646070892, 34.28646028294783, -19.097331116725623,
                            -28.087943162872662},
                           {37.80277123390563, -3.2571969029072276, 112.26918849496327, 66.9347231244047, -40.06618937091002,
                            -54.66780262877968, -9.48861652309627}};
  for (int i = 0; i < 8; ++i) { T.c[i] = cs[i]; T.d[i] = ds[i]; for (int j = 0; j < i; ++j) T.C[i][j] = Cs[i][j]; }
  for (int i = 1; i < 6; ++i) for (int j = 0; j < i; ++j) T.A[i][j] = As[i][j];
  for (int j = 0; j < 5; ++j) { T.A[6][j] = As[5][j]; T.A[7][j] = As[5][j]; T.m[j] = As[5][j]; }
  T.A[6][5] = 1; T.A[7][5] = 1; T.A[7][6] = 1; T.m[5] = 1; T.m[6] = 1; T.m[7] = 1;
  T.beta1 = 0.14; T.beta2 = 0.08; T.rej = 0.14;
  // Continuous extension of order 4, derived for this tableau: the eight tree conditions of order
  // <= 4 of a Rosenbrock method with θ-dependent weights, sum_j b_j(θ) Φ_j(t) = P_t(θ) (P_t(1) =
  // the usual right-hand sides, e.g. θ²/2 - γθ for the second-order tree), are linear in H for the
  // form above and have rank 6 in the 7 non-error stages; one more condition, H u∞ = 0 with u∞
  // the stages of y' = λy as hλ → -∞, makes stiff components interpolate linearly between the
  // step ends instead of being amplified (tight coupling).  Those 7 conditions fix H.
  // (The reference's own Rodas5P interpolant is a different continuous extension.)
  T.ndense = 3;
  const double Hs[3][7] = {
      {16.487964434865184, -2.370717139483559, -36.89699909384169, -47.19777482102162, 29.31762179544809, 37.62133721923128, 6.977388062974808},
      {21.885022549967175, -1.5984168138259751, 162.13711388885017, 126.19157982265247, -76.60482233539331, -106.69765784722038, -28.805926606943324},
      {-15.646484681406143, 3.423681775524067, -62.48695397162234, -48.12822622663184, 30.299848310633063, 44.62468119063477, 18.5833010918263}};
  for (int r = 0; r < 3; ++r) for (int j = 0; j < 7; ++j) T.H[r][j] = Hs[r][j];
  return T;
}

static const Tableau& tableau(int alg) {
  static const Tableau r4 = make_rodas4(), r5 = make_rodas5p();
  return alg == ORC_RODAS5P ? r5 : r4;
}
// gamma of the tableaus (the diagonal of W)
static double tableau_gamma(int alg) { return alg == ORC_RODAS5P ? 0.21193756319429014 : 0.25; }

static bool lu_factor(int n, double* A, int* piv);
static void lu_solve(int n, const double* A, const int* piv, double* b);

// An ODE system with its Rosenbrock linear algebra: w_factor forms and factors W = ihg I - J(t, y)
// and returns ∂f/∂t; w_solve applies W⁻¹ in place.  The defaults use the dense J of jac() and
// dense LU with partial pivoting.
struct OdeSys {
  int n;
  virtual void rhs(double t, const double* y, double* f) = 0;
  virtual void jac(double t, const double* y, double* J, double* ft) = 0;  // J row-major n x n
  virtual bool w_factor(double t, const double* y, double ihg, double* ft) {
    Jd_.resize((size_t)n * n); W_.resize((size_t)n * n); piv_.resize(n);
    jac(t, y, Jd_.data(), ft);
    for (size_t i = 0; i < W_.size(); ++i) W_[i] = -Jd_[i];
    for (int i = 0; i < n; ++i) W_[(size_t)i * n + i] += ihg;
    return lu_factor(n, W_.data(), piv_.data());
  }
  virtual void w_solve(double* b) { lu_solve(n, W_.data(), piv_.data(), b); }
  virtual ~OdeSys() {}
 private:
  std::vector<double> Jd_, W_;
  std::vector<int> piv_;
};
struct StepSink {
  // K: the tableau's dense-output vectors (3 x n) or nullptr (cubic Hermite)
  virtual bool on_step(double t0, const double* y0, const double* f0, double t1, const double* y1, const double* f1,
                       const double* K) = 0;
  virtual ~StepSink() {}
};

static bool lu_factor(int n, double* A, int* piv) {
  for (int k = 0; k < n; ++k) {
    int p = k; double mx = std::fabs(A[k * n + k]);
    for (int i = k + 1; i < n; ++i) { double v = std::fabs(A[i * n + k]); if (v > mx) { mx = v; p = i; } }
    piv[k] = p;
    if (!(mx > 0) || !std::isfinite(mx)) return false;
    if (p != k) for (int j = 0; j < n; ++j) std::swap(A[k * n + j], A[p * n + j]);
    const double inv = 1.0 / A[k * n + k];
    for (int i = k + 1; i < n; ++i) {
      double l = A[i * n + k] * inv; A[i * n + k] = l;
      if (l != 0) for (int j = k + 1; j < n; ++j) A[i * n + j] -= l * A[k * n + j];
    }
  }
  return true;
}
static void lu_solve(int n, const double* A, const int* piv, double* b) {
  for (int k = 0; k < n; ++k) { if (piv[k] != k) std::swap(b[k], b[piv[k]]); }
  for (int i = 0; i < n; ++i) { double s = b[i]; for (int j = 0; j < i; ++j) s -= A[i * n + j] * b[j]; b[i] = s; }
  for (int i = n - 1; i >= 0; --i) { double s = b[i]; for (int j = i + 1; j < n; ++j) s -= A[i * n + j] * b[j]; b[i] = s / A[i * n + i]; }
}

enum { ST_OK = 0, ST_MAXITERS = 1, ST_DTMIN = 2, ST_NONFINITE = 3 };

static int rosenbrock(int alg, OdeSys& sys, double t, double tf, double* y, double rtol, double atol, long maxiters,
                      StepSink* sink, long* nacc, long* nrej) {
  const Tableau& T = tableau(alg);
  const double gam = tableau_gamma(alg);
  const int n = sys.n, S = T.s;
  std::vector<double> f0(n), ft(n), Y(n), F(n), y1(n), f1(n), K(3 * n);
  std::vector<std::vector<double>> U(S, std::vector<double>(n));
  *nacc = 0; *nrej = 0;
  if (!(tf > t)) return ST_OK;
  sys.rhs(t, y, f0.data());
  auto rms = [&](const std::vector<double>& v, const double* yy) {
    double s = 0; for (int i = 0; i < n; ++i) { double sk = atol + std::fabs(yy[i]) * rtol; s += (v[i] / sk) * (v[i] / sk); } return std::sqrt(s / n);
  };
  // initial step (Hairer-Norsett-Wanner II.4)
  double h;
  {
    std::vector<double> yv(y, y + n);
    double d0 = rms(yv, y), d1n = rms(f0, y);
    double h0 = (d0 < 1e-5 || d1n < 1e-5) ? 1e-6 : 0.01 * d0 / d1n;
    h0 = std::min(h0, tf - t);
    for (int i = 0; i < n; ++i) Y[i] = y[i] + h0 * f0[i];
    sys.rhs(t + h0, Y.data(), F.data());
    std::vector<double> df(n); for (int i = 0; i < n; ++i) df[i] = (F[i] - f0[i]) / h0;
    double d2 = rms(df, y);
    double mx = std::max(d1n, d2);
    double h1 = (mx <= 1e-15 || !std::isfinite(mx)) ? std::max(1e-6, h0 * 1e-3) : std::pow(0.01 / mx, 1.0 / 5.0);
    h = std::min(100 * h0, h1);
    if (!std::isfinite(h) || h <= 0) h = 1e-6 * std::max(1.0, std::fabs(t));
  }
  const double kLogErrFloor = std::log(1e-4);  // the controller's floor on errold
  double lerrold = kLogErrFloor; bool last_rejected = false; bool last_nonfinite = false;
  long iters = 0;
  while (t < tf) {
    if (++iters > maxiters) return ST_MAXITERS;
    if (t + h >= tf || t + 1.01 * h >= tf) h = tf - t;
    if (h < 1e-14 * std::max(std::fabs(t), 1e-300) || h <= 0) return last_nonfinite ? ST_NONFINITE : ST_DTMIN;
    const double ihg = 1.0 / (h * gam), ih = 1.0 / h;
    bool ok = sys.w_factor(t, y, ihg, ft.data());
    double err2 = NAN;
    if (ok) {
      for (int st = 0; st < S; ++st) {
        if (st == 0) {
          for (int i = 0; i < n; ++i) U[0][i] = f0[i] + h * T.d[0] * ft[i];
        } else {
          for (int i = 0; i < n; ++i) { double v = y[i]; for (int j = 0; j < st; ++j) v += T.A[st][j] * U[j][i]; Y[i] = v; }
          sys.rhs(t + T.c[st] * h, Y.data(), F.data());
          for (int i = 0; i < n; ++i) {
            double v = 0; for (int j = 0; j < st; ++j) v += T.C[st][j] * U[j][i];
            U[st][i] = F[i] + ih * v + (T.d[st] != 0 ? h * T.d[st] * ft[i] : 0.0);
          }
        }
        sys.w_solve(U[st].data());
      }
      for (int i = 0; i < n; ++i) { double v = y[i]; for (int j = 0; j < S; ++j) v += T.m[j] * U[j][i]; y1[i] = v; }
      double s = 0;
      for (int i = 0; i < n; ++i) {
        double sk = atol + rtol * std::max(std::fabs(y[i]), std::fabs(y1[i]));
        s += (U[S - 1][i] / sk) * (U[S - 1][i] / sk);
      }
      err2 = s / n;  // squared RMS error norm
    }
    const double qmin = 0.2, qmax = 10.0;
    if (std::isfinite(err2) && err2 <= 1.0) {
      const double tnew = (h == tf - t) ? tf : t + h;
      sys.rhs(tnew, y1.data(), f1.data());
      const double* Kp = nullptr;
      if (sink && T.ndense) {
        for (int r = 0; r < T.ndense; ++r)
          for (int i = 0; i < n; ++i) { double v = 0; for (int j = 0; j < S; ++j) v += T.H[r][j] * U[j][i]; K[r * n + i] = v; }
        Kp = K.data();
      }
      if (sink && !sink->on_step(t, y, f0.data(), tnew, y1.data(), f1.data(), Kp)) return ST_OK;
      t = tnew;
      std::memcpy(y, y1.data(), n * sizeof(double));
      f0.swap(f1);
      ++*nacc;
      const double lerr = 0.5 * std::log(std::max(err2, 1e-20));
      double fac = 0.9 * std::exp(-T.beta1 * lerr + T.beta2 * lerrold);
      fac = std::min(qmax, std::max(qmin, fac));
      if (last_rejected) fac = std::min(fac, 1.0);
      lerrold = std::max(lerr, kLogErrFloor);
      h *= fac;
      last_rejected = false; last_nonfinite = false;
    } else {
      ++*nrej;
      last_rejected = true;
      if (!std::isfinite(err2)) { last_nonfinite = true; h *= qmin; }
      else h *= std::max(qmin, 0.9 * std::exp(-0.5 * T.rej * std::log(err2)));
    }
  }
  return ST_OK;
}

// ------------------------------------------------------------------------------------------
// background stage
struct BgSys : OdeSys {
  const Cosmo& P;
  explicit BgSys(const Cosmo& P_) : P(P_) { n = 5; }
  void rhs(double, const double* y, double* f) override { bg_rhs<double>(P, y, f, nullptr); }
  void jac(double, const double* y, double* J, double* ft) override {
    for (int j = 0; j < 5; ++j) {
      Jet<1> yj[5], fj[5];
      for (int i = 0; i < 5; ++i) { yj[i] = Jet<1>(y[i]); }
      yj[j].c[1] = 1.0;
      bg_rhs<Jet<1>>(P, yj, fj, nullptr);
      for (int i = 0; i < 5; ++i) J[i * 5 + j] = fj[i].c[1];
    }
    for (int i = 0; i < 5; ++i) ft[i] = 0;
  }
};

struct Knot { double t, y[5], f[5]; };

struct BgSink : StepSink {
  std::vector<Knot>& knots;
  bool hit = false; double tau0 = 0; double y0[5];
  explicit BgSink(std::vector<Knot>& k) : knots(k) {}
  static void herm(double t0, const double* y0, const double* f0, double t1, const double* y1, const double* f1, double t, double* out) {
    const double h = t1 - t0, s = (t - t0) / h, s2 = s * s, s3 = s2 * s;
    const double h00 = 2 * s3 - 3 * s2 + 1, h10 = s3 - 2 * s2 + s, h01 = -2 * s3 + 3 * s2, h11 = s3 - s2;
    for (int i = 0; i < 5; ++i) out[i] = h00 * y0[i] + h10 * h * f0[i] + h01 * y1[i] + h11 * h * f1[i];
  }
  bool on_step(double t0, const double* y0_, const double* f0, double t1, const double* y1, const double* f1,
               const double*) override {
    if (y1[0] >= 1.0) {  // a = 1 event (src/solve.jl:158-203); root of the step's Hermite interpolant
      double lo = t0, hi = t1, tmp[5];
      for (int it = 0; it < 200; ++it) {
        double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;
        herm(t0, y0_, f0, t1, y1, f1, mid, tmp);
        if (tmp[0] >= 1.0) hi = mid; else lo = mid;
      }
      tau0 = hi; herm(t0, y0_, f0, t1, y1, f1, hi, y0);
      hit = true;
      return false;
    }
    Knot k; k.t = t1; std::memcpy(k.y, y1, sizeof k.y); std::memcpy(k.f, f1, sizeof k.f); knots.push_back(k);
    return true;
  }
};

}  // namespace orc

using namespace orc;

struct orc_bg {
  Cosmo P;
  std::vector<Knot> knots;
  double tau0, kappa0, taurec;
  int status;
  // Hermite spline of the unknowns (src/utils.jl:118-127)
  template <class S> void spline(double tau, S* y) const;       // S = double or Jet<1> (value + d/dtau)
  int interval(double tau) const {
    int lo = 0, hi = (int)knots.size() - 1;
    if (tau <= knots[0].t) return 0;
    if (tau >= knots[hi].t) return hi - 1;
    while (hi - lo > 1) { int mid = (lo + hi) / 2; if (knots[mid].t <= tau) lo = mid; else hi = mid; }
    return lo;
  }
};

template <class S> void orc_bg::spline(double tau, S* y) const {
  const int i = interval(tau);
  const Knot &A = knots[i], &B = knots[i + 1];
  const double h = B.t - A.t, s = (tau - A.t) / h, s2 = s * s, s3 = s2 * s;
  const double h00 = 2 * s3 - 3 * s2 + 1, h10 = s3 - 2 * s2 + s, h01 = -2 * s3 + 3 * s2, h11 = s3 - s2;
  const double d00 = (6 * s2 - 6 * s) / h, d10 = 3 * s2 - 4 * s + 1, d01 = (-6 * s2 + 6 * s) / h, d11 = 3 * s2 - 2 * s;
  for (int j = 0; j < 5; ++j) {
    double v = h00 * A.y[j] + h10 * h * A.f[j] + h01 * B.y[j] + h11 * h * B.f[j];
    double dv = d00 * A.y[j] + d10 * A.f[j] + d01 * B.y[j] + d11 * B.f[j];
    y[j] = S(v);
    if constexpr (!std::is_same<S, double>::value) y[j].c[1] = dv;
  }
}

// Taylor-mode expansion of the background trajectory through the splined state at tau:
// y(tau + s) = sum_k Y_k s^k with (k+1) Y_{k+1} = [f(Y)]_k.  These are the derivatives the
// reference obtains by substituting the background ODE into its symbolic source expressions.
template <int N>
static void bg_taylor(const orc_bg& B, double tau, Jet<N>* y) {
  double y0[5]; B.spline<double>(tau, y0);
  for (int j = 0; j < 5; ++j) y[j] = Jet<N>(y0[j]);
  for (int k = 0; k < N; ++k) {
    Jet<N> f[5]; bg_rhs<Jet<N>>(B.P, y, f, nullptr);
    for (int j = 0; j < 5; ++j) y[j].c[k + 1] = f[j].c[k] / (k + 1);
  }
}

extern "C" int orc_momentum_quadrature(int N, double* x, double* W) { return momentum_quadrature(N, x, W); }

extern "C" orc_bg* orc_bg_solve(const orc_params* p, const orc_model* m, const orc_opts* o, int* status) {
  orc_bg* B = new orc_bg();
  cosmo_init(B->P, p, m, o);
  const Cosmo& P = B->P;
  // initial a from H = 1/tau (src/models/cosmologies.jl:76): tau * a * sqrt(Omega(a)) = 1
  double t0 = P.tau_ini;
  double Orad = P.Og0 + P.On0 + (P.nx > 0 ? P.Oh0 / P.Irho0 * 7 * std::pow(K::PI, 4) / 120 : 0);
  double a = std::sqrt(Orad) * t0;
  for (int it = 0; it < 100; ++it) {
    Jet<1> y[5] = {Jet<1>::var(a), Jet<1>(0.0), Jet<1>(0.0), Jet<1>(1.0), Jet<1>(1.0)}, f[5];
    BgOut<Jet<1>> bo; bg_rhs<Jet<1>>(P, y, f, &bo);
    Jet<1> g = bo.Hc * t0 - 1.0;  // H(a) tau - 1
    double da = -g.c[0] / g.c[1];
    a += da;
    if (std::fabs(da) < 1e-15 * a) break;
  }
  double y[5] = {a, 0.0, 0.0, 1.0, 1.0};
  Knot k0; k0.t = t0; std::memcpy(k0.y, y, sizeof y); bg_rhs<double>(P, y, k0.f, nullptr);
  B->knots.push_back(k0);
  BgSys sys(P);
  BgSink sink(B->knots);
  long na, nr;
  int st = rosenbrock(P.alg_bg, sys, t0, P.tau_max, y, P.rtol_bg, P.atol_bg, P.maxiters, &sink, &na, &nr);
  if (!sink.hit || st != ST_OK || !std::isfinite(a)) {
    B->status = st ? st : ST_NONFINITE; *status = B->status;
    B->tau0 = B->kappa0 = B->taurec = NAN;
    return B;
  }
  Knot kn; kn.t = sink.tau0; std::memcpy(kn.y, sink.y0, sizeof kn.y); bg_rhs<double>(P, kn.y, kn.f, nullptr);
  B->knots.push_back(kn);
  // Knot slopes of the stiff recombination unknowns (dT, XH+, XHe+).  Their right-hand sides
  // multiply rounding-level departures from quasi-equilibrium by huge rates, so the spline takes
  // smooth slopes instead: the derivative of the local 5-knot interpolating polynomial.  (The
  // reference likewise uses the derivative of its integrator's dense output, src/utils.jl:123.)
  {
    const int nk = (int)B->knots.size();
    std::vector<double> d(3 * nk);
    // stencils exclude knot 0: the initial condition dT = 0 is off quasi-equilibrium and the first
    // knots resolve a ~1e-14-wide transient that must not leak into the slopes
    for (int i = 0; i < nk; ++i) {
      int lo = std::max(1, std::min(i - 2, nk - 5)), hi = std::min(nk - 1, lo + 4);
      const double xi = B->knots[i].t;
      for (int c = 0; c < 3; ++c) d[3 * i + c] = 0;
      for (int j = lo; j <= hi; ++j) {
        const double xj = B->knots[j].t;
        double w;
        if (j == i) { w = 0; for (int m = lo; m <= hi; ++m) if (m != i) w += 1 / (xi - B->knots[m].t); }
        else {
          double num = 1, den = 1;
          for (int m = lo; m <= hi; ++m) { if (m == j) continue; den *= (xj - B->knots[m].t); if (m != i) num *= (xi - B->knots[m].t); }
          w = num / den;
        }
        for (int c = 0; c < 3; ++c) d[3 * i + c] += w * B->knots[j].y[2 + c];
      }
    }
    for (int i = 0; i < nk; ++i) for (int c = 0; c < 3; ++c) B->knots[i].f[2 + c] = d[3 * i + c];
  }
  B->tau0 = sink.tau0;
  B->kappa0 = kn.y[1];
  // recombination time: maximum of the visibility function v = -kappa' exp(-kappa)
  auto vis = [&](double tau) {
    double yy[5], ff[5]; B->spline<double>(tau, yy); bg_rhs<double>(P, yy, ff, nullptr);
    return -ff[1] * std::exp(-(yy[1] - B->kappa0));
  };
  int imax = 0; double vmax = -1;
  for (size_t i = 0; i < B->knots.size(); ++i) { double v = vis(B->knots[i].t); if (v > vmax) { vmax = v; imax = (int)i; } }
  double lo = B->knots[std::max(imax - 1, 0)].t, hi = B->knots[std::min<size_t>(imax + 1, B->knots.size() - 1)].t;
  const double gr = 0.5 * (std::sqrt(5.0) - 1);
  double x1 = hi - gr * (hi - lo), x2 = lo + gr * (hi - lo), v1 = vis(x1), v2 = vis(x2);
  for (int it = 0; it < 200 && hi - lo > 1e-15 * hi; ++it) {
    if (v1 > v2) { hi = x2; x2 = x1; v2 = v1; x1 = hi - gr * (hi - lo); v1 = vis(x1); }
    else { lo = x1; x1 = x2; v1 = v2; x2 = lo + gr * (hi - lo); v2 = vis(x2); }
  }
  B->taurec = 0.5 * (lo + hi);
  B->status = ST_OK; *status = ST_OK;
  return B;
}

extern "C" void orc_bg_free(orc_bg* b) { delete b; }
extern "C" int orc_bg_nknots(const orc_bg* b) { return (int)b->knots.size(); }
extern "C" void orc_bg_knots(const orc_bg* b, double* tau, double* y) {
  for (size_t i = 0; i < b->knots.size(); ++i) { tau[i] = b->knots[i].t; for (int j = 0; j < 5; ++j) y[i * 5 + j] = b->knots[i].y[j]; }
}
extern "C" void orc_bg_info(const orc_bg* b, double* info) {
  const Cosmo& P = b->P;
  double v[] = {b->tau0, b->kappa0, b->taurec, P.Og0, P.On0, P.Oh0, P.OL0, (double)b->knots.size(), P.fHe, P.As, P.kpivot, P.y0, P.Irho0};
  std::memcpy(info, v, sizeof v);
}
extern "C" void orc_bg_eval(const orc_bg* b, int n, const double* tau, double* out) {
  for (int i = 0; i < n; ++i) {
    Jet<2> y[5], f[5]; bg_taylor<2>(*b, tau[i], y);
    BgOut<Jet<2>> o; bg_rhs<Jet<2>>(b->P, y, f, &o);
    Jet<2> kap = y[1] - b->kappa0;
    Jet<2> v = -o.kd * exp(-kap);
    double r[10] = {o.a.c[0], o.Hc.c[0], o.kd.c[0], kap.c[0], v.c[0], v.c[1], o.cs2.c[0], o.Xe.c[0], o.Tb.c[0], o.XHepp.c[0]};
    std::memcpy(out + 10 * i, r, sizeof r);
  }
}

// ------------------------------------------------------------------------------------------
// perturbation stage
namespace orc {

struct PtLayout {
  int Lg, Ln, Lh, nx, n;
  int Phi = 0, dc = 1, tc = 2, db = 3, tb = 4;
  int F(int l) const { return 5 + l; }
  int G(int l) const { return 5 + (Lg + 1) + l; }
  int N(int l) const { return 5 + 2 * (Lg + 1) + l; }
  int H(int i, int l) const { return 5 + 2 * (Lg + 1) + (Ln + 1) + i * (Lh + 1) + l; }
  explicit PtLayout(const Cosmo& P) : Lg(P.Lg), Ln(P.Ln), Lh(P.Lh), nx(P.nx) { n = 5 + 2 * (Lg + 1) + (Ln + 1) + nx * (Lh + 1); }
};

// time-dependent background coefficients of the (linear) perturbation equations
template <class S> struct PtCoef { S a, Hc, kd, cs2, tau; };

template <class S>
static void pt_psi_phidot(const Cosmo& P, const PtLayout& L, double k, const PtCoef<S>& C, S* pPsi, S* pPhid) {
  // Psi = Phi - 12 pi a^2 Pi / k^2           (src/models/gravity.jl:39, src/models/cosmologies.jl:94)
  // Phi' = -4pi/3 a^2/H dRho - k^2/(3H) Phi - H Psi   (src/models/gravity.jl:38)
  const int n = L.n;
  for (int i = 0; i < n; ++i) { pPsi[i] = S(0.0); pPhid[i] = S(0.0); }
  const S ia2 = 1.0 / (C.a * C.a);
  const S ia = 1.0 / C.a;
  const double ik2 = 1.0 / (k * k);
  pPsi[L.Phi] = S(1.0);
  pPsi[L.F(2)] = -3.0 * ik2 * P.Og0 * ia2;
  pPsi[L.N(2)] = -3.0 * ik2 * P.On0 * ia2;
  const S m2H = -0.5 / C.Hc;
  pPhid[L.dc] = m2H * P.Oc0 * ia;
  pPhid[L.db] = m2H * P.Ob0 * ia;
  pPhid[L.F(0)] = m2H * P.Og0 * ia2;
  pPhid[L.N(0)] = m2H * P.On0 * ia2;
  if (P.nx > 0) {
    const double wh = P.Oh0 / P.Irho0;
    for (int i = 0; i < P.nx; ++i) {
      const S E = sqrt(P.xq[i] * P.xq[i] + (P.y0 * P.y0) * (C.a * C.a));
      pPsi[L.H(i, 2)] = -3.0 * ik2 * wh * ia2 * P.Wq[i] * P.xq[i] * P.xq[i] / E;
      pPhid[L.H(i, 0)] = m2H * wh * ia2 * P.Wq[i] * E;
    }
  }
  pPhid[L.Phi] = pPhid[L.Phi] - k * k / (3.0 * C.Hc);
  for (int i = 0; i < n; ++i) pPhid[i] = pPhid[i] - C.Hc * pPsi[i];
}

// J(tau) of the linear system u' = J(tau) u, written through an accumulator: acc.add(r, c, v) adds
// v to J[r][c], acc.addv(r, s, v) adds s * v (a functional's weight vector, pPsi or pPhid) to row r.
template <class S, class Acc>
static void pt_assemble(const Cosmo& P, const PtLayout& L, double k, const PtCoef<S>& C, Acc& acc, S* pPsi, S* pPhid) {
  pt_psi_phidot(P, L, k, C, pPsi, pPhid);
  struct RowRef {
    Acc& a; int r;
    struct Cell { Acc& a; int r, c; void operator+=(const S& v) { a.add(r, c, v); } };
    Cell operator[](int c) { return Cell{a, r, c}; }
  };
  auto row = [&](int r) { return RowRef{acc, r}; };
  auto addv = [&](int r, double s, const S* v) { acc.addv(r, S(s), v); };
  auto addvS = [&](int r, const S& s, const S* v) { acc.addv(r, s, v); };
  const S kd = C.kd, Hc = C.Hc;
  // metric
  addv(L.Phi, 1.0, pPhid);
  // CDM (src/models/generic_species.jl:46-47 with w = cs2 = 0)
  row(L.dc)[L.tc] += -1.0; addv(L.dc, 3.0, pPhid);
  row(L.tc)[L.tc] += -Hc; addv(L.tc, k * k, pPsi);
  // baryons (cs2 thermal; momentum exchange src/models/cosmologies.jl:95)
  const S R = (4.0 / 3.0) * (P.Og0 / P.Ob0) / C.a;
  row(L.db)[L.tb] += -1.0; row(L.db)[L.db] += -3.0 * Hc * C.cs2; addv(L.db, 3.0, pPhid);
  row(L.tb)[L.tb] += -Hc + kd * R; row(L.tb)[L.db] += C.cs2 * k * k; addv(L.tb, k * k, pPsi);
  row(L.tb)[L.F(1)] += -kd * R * (0.75 * k);
  // photons (src/models/photons.jl:28-60), Pi = F2 + G0 + G2
  const int Lg = P.Lg;
  row(L.F(0))[L.F(1)] += -k; addv(L.F(0), 4.0, pPhid);
  row(L.F(1))[L.F(0)] += k / 3; row(L.F(1))[L.F(2)] += -2 * k / 3; addv(L.F(1), 4 * k / 3, pPsi);
  row(L.F(1))[L.tb] += -(4.0 / 3.0) * kd / k; row(L.F(1))[L.F(1)] += kd;
  for (int l = 2; l < Lg; ++l) {
    auto Rw = row(L.F(l));
    Rw[L.F(l - 1)] += k * l / (2.0 * l + 1); Rw[L.F(l + 1)] += -k * (l + 1) / (2.0 * l + 1); Rw[L.F(l)] += kd;
    if (l == 2) { Rw[L.F(2)] += -kd / 10; Rw[L.G(0)] += -kd / 10; Rw[L.G(2)] += -kd / 10; }
  }
  row(L.F(Lg))[L.F(Lg - 1)] += k; row(L.F(Lg))[L.F(Lg)] += -(Lg + 1) / C.tau + kd;
  row(L.G(0))[L.G(1)] += -k; row(L.G(0))[L.G(0)] += kd;
  row(L.G(0))[L.F(2)] += -kd / 2; row(L.G(0))[L.G(0)] += -kd / 2; row(L.G(0))[L.G(2)] += -kd / 2;
  row(L.G(1))[L.G(0)] += k / 3; row(L.G(1))[L.G(2)] += -2 * k / 3; row(L.G(1))[L.G(1)] += kd;
  for (int l = 2; l < Lg; ++l) {
    auto Rw = row(L.G(l));
    Rw[L.G(l - 1)] += k * l / (2.0 * l + 1); Rw[L.G(l + 1)] += -k * (l + 1) / (2.0 * l + 1); Rw[L.G(l)] += kd;
    if (l == 2) { Rw[L.F(2)] += -kd / 10; Rw[L.G(0)] += -kd / 10; Rw[L.G(2)] += -kd / 10; }
  }
  row(L.G(Lg))[L.G(Lg - 1)] += k; row(L.G(Lg))[L.G(Lg)] += -(Lg + 1) / C.tau + kd;
  // massless neutrinos (src/models/neutrinos.jl:22-26)
  const int Ln = P.Ln;
  row(L.N(0))[L.N(1)] += -k; addv(L.N(0), 4.0, pPhid);
  row(L.N(1))[L.N(0)] += k / 3; row(L.N(1))[L.N(2)] += -2 * k / 3; addv(L.N(1), 4 * k / 3, pPsi);
  for (int l = 2; l < Ln; ++l) { auto Rw = row(L.N(l)); Rw[L.N(l - 1)] += k * l / (2.0 * l + 1); Rw[L.N(l + 1)] += -k * (l + 1) / (2.0 * l + 1); }
  row(L.N(Ln))[L.N(Ln - 1)] += k; row(L.N(Ln))[L.N(Ln)] += -(Ln + 1) / C.tau;
  // massive neutrinos (src/models/neutrinos.jl:129-132)
  const int Lh = P.Lh;
  for (int i = 0; i < P.nx; ++i) {
    const S E = sqrt(P.xq[i] * P.xq[i] + (P.y0 * P.y0) * (C.a * C.a));
    const S q = P.xq[i] / E;
    const double dl = P.dlnf[i];
    row(L.H(i, 0))[L.H(i, 1)] += -k * q; addv(L.H(i, 0), -dl, pPhid);
    row(L.H(i, 1))[L.H(i, 0)] += (k / 3) * q; row(L.H(i, 1))[L.H(i, 2)] += -(2 * k / 3) * q;
    addvS(L.H(i, 1), -(k / 3) * dl / q, pPsi);
    for (int l = 2; l < Lh; ++l) {
      auto Rw = row(L.H(i, l));
      Rw[L.H(i, l - 1)] += k * q * (l / (2.0 * l + 1)); Rw[L.H(i, l + 1)] += -k * q * ((l + 1) / (2.0 * l + 1));
    }
    row(L.H(i, Lh))[L.H(i, Lh - 1)] += k * q; row(L.H(i, Lh))[L.H(i, Lh)] += -(Lh + 1) / C.tau;
  }
}

template <class S> struct DenseAcc {
  S* J; int n;
  void add(int r, int c, const S& v) { J[(size_t)r * n + c] += v; }
  void addv(int r, const S& s, const S* v) { S* R = J + (size_t)r * n; for (int i = 0; i < n; ++i) R[i] += s * v[i]; }
};

// Dense J(tau) (the checker's form).
template <class S>
static void pt_jacobian(const Cosmo& P, const PtLayout& L, double k, const PtCoef<S>& C, S* J, S* pPsi, S* pPhid) {
  const int n = L.n;
  for (int i = 0; i < n * n; ++i) J[i] = S(0.0);
  DenseAcc<S> acc{J, n};
  pt_assemble<S>(P, L, k, C, acc, pPsi, pPhid);
}

// background coefficients from the spline (values, plus d/dtau through the spline for Jet<1>)
template <class S>
static void pt_coef_spline(const orc_bg& B, double tau, PtCoef<S>& C) {
  S y[5], f[5]; B.spline<S>(tau, y);
  BgOut<S> o; bg_rhs<S>(B.P, y, f, &o);
  C.a = o.a; C.Hc = o.Hc; C.kd = o.kd; C.cs2 = o.cs2;
  if constexpr (std::is_same<S, double>::value) C.tau = tau; else C.tau = S::var(tau);
}

struct PtSys : OdeSys {
  const orc_bg& B; const Cosmo& P; PtLayout L; double k;
  std::vector<double> pPsi, pPhid; std::vector<Jet<1>> Jj, pPsij, pPhidj;
  PtSys(const orc_bg& B_, double k_) : B(B_), P(B_.P), L(B_.P), k(k_) {
    n = L.n; pPsi.resize(n); pPhid.resize(n); Jj.resize((size_t)n * n); pPsij.resize(n); pPhidj.resize(n);
  }
  std::vector<double> Jd;
  void rhs(double t, const double* y, double* f) override {
    PtCoef<double> C; pt_coef_spline<double>(B, t, C);
    Jd.resize((size_t)n * n);
    pt_jacobian<double>(P, L, k, C, Jd.data(), pPsi.data(), pPhid.data());
    for (int i = 0; i < n; ++i) { double s = 0; const double* R = &Jd[(size_t)i * n]; for (int j = 0; j < n; ++j) s += R[j] * y[j]; f[i] = s; }
  }
  // f = J y and g = J' y + J f with the coefficients C (value and τ-derivative); fills pPsij
  virtual void source_products(const PtCoef<Jet<1>>& C, const double* y, double* f, double* g) {
    pt_jacobian<Jet<1>>(P, L, k, C, Jj.data(), pPsij.data(), pPhidj.data());
    for (int i = 0; i < n; ++i) { double s = 0; for (int j = 0; j < n; ++j) s += Jj[(size_t)i * n + j].c[0] * y[j]; f[i] = s; }
    for (int i = 0; i < n; ++i) {
      double s = 0;
      for (int j = 0; j < n; ++j) s += Jj[(size_t)i * n + j].c[1] * y[j] + Jj[(size_t)i * n + j].c[0] * f[j];
      g[i] = s;
    }
  }
  void jac(double t, const double* y, double* J, double* ft) override {
    PtCoef<Jet<1>> C; pt_coef_spline<Jet<1>>(B, t, C);
    pt_jacobian<Jet<1>>(P, L, k, C, Jj.data(), pPsij.data(), pPhidj.data());
    for (int i = 0; i < n; ++i) {
      double s = 0;
      for (int j = 0; j < n; ++j) { const Jet<1>& e = Jj[(size_t)i * n + j]; J[(size_t)i * n + j] = e.c[0]; s += e.c[1] * y[j]; }
      ft[i] = s;
    }
  }
};

// ------------------------------------------------------------------------------------------
// Sparse linear algebra of the CPU baseline (the reference's path: Rodas5P with a sparse LU of
// W = I/(hγ) - J, KLU in LinearSolve.jl, src/solve.jl:314-317,327-341).  The dense PtSys above is
// the checker; this one does the same arithmetic on the structural nonzeros only:
//   * J is assembled into its nonzero slots (pattern found once per model from the dense form at
//     generic times) and applied as a sparse product;
//   * W is permuted symmetrically by a minimum-degree order of its pattern and factored by
//     right-looking elimination with threshold partial pivoting (the diagonal is kept while it is at
//     least a tenth of the column's largest entry), visiting only nonzero multipliers and the pivot
//     row's nonzeros; the solves use the recorded L columns and U rows.
struct SparsePattern {
  int n = 0;
  std::vector<int> slot;         // n*n -> index of the nonzero, or -1
  std::vector<int> row, col;     // per nonzero
  std::vector<int> fidx;         // components carrying a Ψ or Φ̇ weight
  std::vector<int> perm, iperm;  // elimination order: position p holds component perm[p]
};

static void build_sparse_pattern(const orc_bg& B, SparsePattern& SP) {
  const Cosmo& P = B.P; PtLayout L(P);
  const int n = L.n;
  SP.n = n;
  std::vector<char> nz((size_t)n * n, 0), fz(n, 0);
  std::vector<double> J((size_t)n * n), pPsi(n), pPhid(n);
  const double t0 = B.knots.front().t, t1 = B.tau0;
  const double ts[3] = {t0 * 1.37, std::sqrt(t0 * t1) * 0.91, t1 * 0.73};
  for (double k : {1.37, 171.3}) {
    for (double tau : ts) {
      PtCoef<double> C; pt_coef_spline<double>(B, tau, C);
      pt_jacobian<double>(P, L, k, C, J.data(), pPsi.data(), pPhid.data());
      for (size_t e = 0; e < J.size(); ++e) if (J[e] != 0) nz[e] = 1;
      for (int i = 0; i < n; ++i) if (pPsi[i] != 0 || pPhid[i] != 0) fz[i] = 1;
    }
  }
  for (int i = 0; i < n; ++i) nz[(size_t)i * n + i] = 1;  // W's diagonal
  SP.slot.assign((size_t)n * n, -1);
  SP.row.clear(); SP.col.clear(); SP.fidx.clear();
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c)
      if (nz[(size_t)r * n + c]) { SP.slot[(size_t)r * n + c] = (int)SP.row.size(); SP.row.push_back(r); SP.col.push_back(c); }
  for (int i = 0; i < n; ++i) if (fz[i]) SP.fidx.push_back(i);
  // rows that take a functional get every functional column (the assembly adds the whole vector)
  // minimum-degree order on the symmetrised pattern
  std::vector<std::vector<char>> adj(n, std::vector<char>(n, 0));
  for (size_t e = 0; e < SP.row.size(); ++e) {
    const int r = SP.row[e], c = SP.col[e];
    if (r != c) { adj[r][c] = 1; adj[c][r] = 1; }
  }
  std::vector<char> done(n, 0);
  SP.perm.clear();
  for (int step = 0; step < n; ++step) {
    int best = -1, bdeg = 1 << 30;
    for (int v = 0; v < n; ++v) {
      if (done[v]) continue;
      int d = 0; for (int u = 0; u < n; ++u) d += (!done[u] && adj[v][u]);
      if (d < bdeg) { bdeg = d; best = v; }
    }
    done[best] = 1; SP.perm.push_back(best);
    std::vector<int> nb;
    for (int u = 0; u < n; ++u) if (!done[u] && adj[best][u]) nb.push_back(u);
    for (int a : nb) for (int b : nb) if (a != b) adj[a][b] = 1;
  }
  SP.iperm.assign(n, 0);
  for (int p = 0; p < n; ++p) SP.iperm[SP.perm[p]] = p;
}

template <class S> struct SparseAcc {
  const SparsePattern& P; S* v;
  void add(int r, int c, const S& x) { v[P.slot[(size_t)r * P.n + c]] += x; }
  void addv(int r, const S& s, const S* w) {
    for (int i : P.fidx) { const int sl = P.slot[(size_t)r * P.n + i]; if (sl >= 0) v[sl] += s * w[i]; }
  }
};

struct SparsePtSys : PtSys {
  const SparsePattern& SP;
  std::vector<double> vals, A, dinv;
  std::vector<Jet<1>> jvals, sv;
  std::vector<int> piv, lptr, lidx, uptr, uidx, rows, ucols;
  std::vector<double> lval, uval, work;
  int nwords;
  std::vector<uint64_t> rowbits, colbits;
  SparsePtSys(const orc_bg& B_, double k_, const SparsePattern& sp) : PtSys(B_, k_), SP(sp) {
    const size_t nnz = SP.row.size();
    vals.resize(nnz); jvals.resize(nnz); sv.resize(nnz); A.assign((size_t)n * n, 0.0); dinv.resize(n); piv.resize(n); work.resize(n);
    nwords = (n + 63) / 64;
    rowbits.assign((size_t)n * nwords, 0); colbits.assign((size_t)n * nwords, 0);
  }
  void rhs(double t, const double* y, double* f) override {
    PtCoef<double> C; pt_coef_spline<double>(B, t, C);
    std::fill(vals.begin(), vals.end(), 0.0);
    SparseAcc<double> acc{SP, vals.data()};
    pt_assemble<double>(P, L, k, C, acc, pPsi.data(), pPhid.data());
    for (int i = 0; i < n; ++i) f[i] = 0;
    for (size_t e = 0; e < vals.size(); ++e) f[SP.row[e]] += vals[e] * y[SP.col[e]];
  }
  bool w_factor(double t, const double* y, double ihg, double* ft) override {
    PtCoef<Jet<1>> C; pt_coef_spline<Jet<1>>(B, t, C);
    std::fill(jvals.begin(), jvals.end(), Jet<1>(0.0));
    SparseAcc<Jet<1>> acc{SP, jvals.data()};
    pt_assemble<Jet<1>>(P, L, k, C, acc, pPsij.data(), pPhidj.data());
    for (int i = 0; i < n; ++i) ft[i] = 0;
    for (size_t e = 0; e < jvals.size(); ++e) ft[SP.row[e]] += jvals[e].c[1] * y[SP.col[e]];
    // W in elimination order.  Row and column bitmaps track the nonzeros (pattern + fill), so the
    // elimination touches nonzeros only; clear what the previous factorisation left.
    const int nw = nwords;
    for (int i = 0; i < n; ++i) {
      uint64_t* rb = &rowbits[(size_t)i * nw];
      for (int w = 0; w < nw; ++w) {
        for (uint64_t b = rb[w]; b; b &= b - 1) A[(size_t)i * n + 64 * w + __builtin_ctzll(b)] = 0.0;
        rb[w] = 0;
      }
    }
    std::fill(colbits.begin(), colbits.end(), 0);
    auto setbit = [&](int i, int j) {
      rowbits[(size_t)i * nw + (j >> 6)] |= 1ull << (j & 63);
      colbits[(size_t)j * nw + (i >> 6)] |= 1ull << (i & 63);
    };
    for (size_t e = 0; e < jvals.size(); ++e) {
      const int r = SP.iperm[SP.row[e]], c = SP.iperm[SP.col[e]];
      A[(size_t)r * n + c] -= jvals[e].c[0];
      setbit(r, c);
    }
    for (int i = 0; i < n; ++i) { A[(size_t)i * n + i] += ihg; setbit(i, i); }
    lptr.assign(1, 0); uptr.assign(1, 0); lidx.clear(); lval.clear(); uidx.clear(); uval.clear();
    for (int kk = 0; kk < n; ++kk) {
      // candidate pivots: nonzero rows of column kk at or below the diagonal
      rows.clear();
      double mx = 0; int pbest = -1;
      const uint64_t* cb = &colbits[(size_t)kk * nw];
      for (int w = kk >> 6; w < nw; ++w) {
        uint64_t b = cb[w];
        if (w == (kk >> 6)) b &= ~0ull << (kk & 63);
        for (; b; b &= b - 1) {
          const int i = 64 * w + __builtin_ctzll(b);
          const double a = std::fabs(A[(size_t)i * n + kk]);
          rows.push_back(i);
          if (a > mx) { mx = a; pbest = i; }
        }
      }
      if (!(mx > 0) || !std::isfinite(mx)) return false;
      int p = kk;
      if (!(std::fabs(A[(size_t)kk * n + kk]) >= 0.1 * mx)) p = pbest;
      piv[kk] = p;
      if (p != kk) {  // swap rows kk and p over their nonzero columns, and the bitmaps with them
        uint64_t* ra = &rowbits[(size_t)kk * nw];
        uint64_t* rp = &rowbits[(size_t)p * nw];
        for (int w = 0; w < nw; ++w) {
          for (uint64_t b = ra[w] | rp[w]; b; b &= b - 1) {
            const int j = 64 * w + __builtin_ctzll(b);
            std::swap(A[(size_t)kk * n + j], A[(size_t)p * n + j]);
            uint64_t* c = &colbits[(size_t)j * nw];
            const bool bk = (c[kk >> 6] >> (kk & 63)) & 1, bp = (c[p >> 6] >> (p & 63)) & 1;
            if (bk != bp) { c[kk >> 6] ^= 1ull << (kk & 63); c[p >> 6] ^= 1ull << (p & 63); }
          }
          std::swap(ra[w], rp[w]);
        }
        for (int& r : rows) if (r == p) r = kk; else if (r == kk) r = p;
      }
      const double d = 1.0 / A[(size_t)kk * n + kk];
      dinv[kk] = d;
      ucols.clear();
      const uint64_t* rk = &rowbits[(size_t)kk * nw];
      for (int w = kk >> 6; w < nw; ++w) {
        uint64_t b = rk[w];
        if (w == (kk >> 6)) b &= (kk & 63) == 63 ? 0 : ~0ull << ((kk & 63) + 1);
        for (; b; b &= b - 1) {
          const int j = 64 * w + __builtin_ctzll(b);
          ucols.push_back(j); uidx.push_back(j); uval.push_back(A[(size_t)kk * n + j]);
        }
      }
      uptr.push_back((int)uidx.size());
      const double* Rk = &A[(size_t)kk * n];
      for (int i : rows) {
        if (i == kk) continue;
        const double l = A[(size_t)i * n + kk] * d;
        lidx.push_back(i); lval.push_back(l);
        double* Ri = &A[(size_t)i * n];
        uint64_t* ri = &rowbits[(size_t)i * nw];
        for (int j : ucols) {
          Ri[j] -= l * Rk[j];
          if (!((ri[j >> 6] >> (j & 63)) & 1)) setbit(i, j);
        }
      }
      lptr.push_back((int)lidx.size());
    }
    return true;
  }
  void source_products(const PtCoef<Jet<1>>& C, const double* y, double* f, double* g) override {
    std::fill(sv.begin(), sv.end(), Jet<1>(0.0));
    SparseAcc<Jet<1>> acc{SP, sv.data()};
    pt_assemble<Jet<1>>(P, L, k, C, acc, pPsij.data(), pPhidj.data());
    for (int i = 0; i < n; ++i) { f[i] = 0; g[i] = 0; }
    for (size_t e = 0; e < sv.size(); ++e) f[SP.row[e]] += sv[e].c[0] * y[SP.col[e]];
    for (size_t e = 0; e < sv.size(); ++e) g[SP.row[e]] += sv[e].c[1] * y[SP.col[e]] + sv[e].c[0] * f[SP.col[e]];
  }
  void w_solve(double* b) override {
    double* x = work.data();
    for (int i = 0; i < n; ++i) x[SP.iperm[i]] = b[i];
    for (int kk = 0; kk < n; ++kk) {
      if (piv[kk] != kk) std::swap(x[kk], x[piv[kk]]);
      const double xk = x[kk];
      for (int e = lptr[kk]; e < lptr[kk + 1]; ++e) x[lidx[e]] -= lval[e] * xk;
    }
    for (int kk = n - 1; kk >= 0; --kk) {
      double v = x[kk];
      for (int e = uptr[kk]; e < uptr[kk + 1]; ++e) v -= uval[e] * x[uidx[e]];
      x[kk] = v * dinv[kk];
    }
    for (int i = 0; i < n; ++i) b[i] = x[SP.iperm[i]];
  }
};

// adiabatic initial conditions (src/models/cosmologies.jl:74-77, photons.jl:47-67,
// neutrinos.jl:33-39,134-139, generic_species.jl:54-57); Phi from the shear constraint.
static void pt_initial(const orc_bg& B, double k, double tau, double* y, double* extra) {
  const Cosmo& P = B.P; PtLayout L(P);
  const int n = L.n;
  for (int i = 0; i < n; ++i) y[i] = 0;
  double yb[5], fb[5]; B.spline<double>(tau, yb);
  BgOut<double> o; bg_rhs<double>(P, yb, fb, &o);
  const double a = o.a, kd = o.kd;
  const double ia4 = 1 / (a * a * a * a);
  double rg = P.Og0 * ia4, rn = P.On0 * ia4, rh = 0;
  if (P.nx > 0) { double Ir = 0; for (int i = 0; i < P.nx; ++i) Ir += P.Wq[i] * std::sqrt(P.xq[i] * P.xq[i] + P.y0 * P.y0 * a * a); rh = P.Oh0 / P.Irho0 * Ir * ia4; }
  const double fnu = (rn + rh) / (rg + rn + rh);
  const double C = 0.5;
  const double Psi = 20 * C / (15 + 4 * fnu);
  const double kt = k * tau;
  y[L.dc] = -1.5 * Psi; y[L.tc] = 0.5 * k * kt * Psi;
  y[L.db] = -1.5 * Psi; y[L.tb] = 0.5 * k * kt * Psi;
  y[L.F(0)] = -2 * Psi;
  y[L.F(1)] = 2.0 / 3.0 * kt * Psi;
  y[L.F(2)] = -8.0 / 15.0 * k / kd * y[L.F(1)];
  y[L.F(3)] = -3.0 / 7.0 * k / kd * y[L.F(2)];
  y[L.G(0)] = 5.0 / 16.0 * y[L.F(2)];
  y[L.G(1)] = -1.0 / 16.0 * k / kd * y[L.F(2)];
  y[L.G(2)] = 1.0 / 16.0 * y[L.F(2)];
  y[L.G(3)] = -3.0 / 7.0 * k / kd * y[L.G(2)];
  y[L.N(0)] = -2 * Psi;
  y[L.N(1)] = 4.0 / (3.0 * k) * (0.5 * k * kt * Psi);
  y[L.N(2)] = 2 * (1.0 / 15.0) * kt * kt * Psi;
  y[L.N(3)] = 3.0 / 7.0 * kt * y[L.N(2)];
  for (int i = 0; i < P.nx; ++i) {
    const double E = std::sqrt(P.xq[i] * P.xq[i] + P.y0 * P.y0 * a * a), dl = P.dlnf[i];
    y[L.H(i, 0)] = -0.25 * (-2 * Psi) * dl;
    y[L.H(i, 1)] = -1.0 / 3.0 * E / P.xq[i] * (0.5 * kt * Psi) * dl;
    y[L.H(i, 2)] = -0.5 * (1.0 / 15.0 * kt * kt * Psi) * dl;
  }
  // Phi: k^2 (Phi - Psi) = 12 pi a^2 Pi with Pi from the initial shears
  PtCoef<double> Cf; Cf.a = a; Cf.Hc = o.Hc; Cf.kd = kd; Cf.cs2 = o.cs2; Cf.tau = tau;
  std::vector<double> pPsi(n), pPhid(n);
  pt_psi_phidot<double>(P, L, k, Cf, pPsi.data(), pPhid.data());
  double shear = 0; for (int i = 0; i < n; ++i) if (i != L.Phi) shear += pPsi[i] * y[i];
  y[L.Phi] = Psi - shear;  // Psi = Phi + shear
  if (extra) { extra[0] = y[L.Phi]; extra[1] = Psi; extra[2] = fnu; }
}

struct PtSink : StepSink {
  PtSys& S; int ntau; const double* taus; int mode; double* out; int next = 0;
  std::vector<double> yi;
  PtSink(PtSys& s, int nt, const double* ts, int md, double* o) : S(s), ntau(nt), taus(ts), mode(md), out(o) { yi.resize(s.n); }
  void emit(int it, double tau, const double* y);
  bool on_step(double t0, const double* y0, const double* f0, double t1, const double* y1, const double* f1,
               const double* K) override {
    const int n = S.n;
    while (next < ntau && taus[next] <= t1) {
      const double tau = taus[next];
      if (tau < t0) { emit(next, tau, nullptr); ++next; continue; }
      const double h = t1 - t0, s = (tau - t0) / h, s2 = s * s, s3 = s2 * s;
      if (K) {
        const double s1 = 1 - s;
        for (int i = 0; i < n; ++i) yi[i] = s1 * y0[i] + s * (y1[i] + s1 * (K[i] + s * (K[n + i] + s * K[2 * n + i])));
      } else {
        const double h00 = 2 * s3 - 3 * s2 + 1, h10 = s3 - 2 * s2 + s, h01 = -2 * s3 + 3 * s2, h11 = s3 - s2;
        for (int i = 0; i < n; ++i) yi[i] = h00 * y0[i] + h10 * h * f0[i] + h01 * y1[i] + h11 * h * f1[i];
      }
      emit(next, tau, yi.data());
      ++next;
    }
    return true;
  }
};

// line-of-sight sources (src/models/cosmologies.jl:99-105) at tau for state y
static void pt_sources(PtSys& S, double tau, const double* y, double* src) {
  const orc_bg& B = S.B; const Cosmo& P = B.P; const PtLayout& L = S.L; const double k = S.k; const int n = L.n;
  // background jets (Taylor-mode through the splined state)
  Jet<3> yb[5], fb[5]; bg_taylor<3>(B, tau, yb);
  BgOut<Jet<3>> o; bg_rhs<Jet<3>>(P, yb, fb, &o);
  const Jet<3> ekap = exp(-(yb[1] - B.kappa0));
  const Jet<3> v = -o.kd * ekap;
  const double V = v.c[0], Vd = v.c[1], Vdd = 2 * v.c[2], Ek = ekap.c[0];
  PtCoef<Jet<1>> C;
  auto t1 = [](const Jet<3>& x) { Jet<1> r; r.c[0] = x.c[0]; r.c[1] = x.c[1]; return r; };
  C.a = t1(o.a); C.Hc = t1(o.Hc); C.kd = t1(o.kd); C.cs2 = t1(o.cs2); C.tau = Jet<1>::var(tau);
  std::vector<double> f(n), g(n);
  S.source_products(C, y, f.data(), g.data());  // f = J y, g = J' y + J f; S.pPsij holds Ψ's weights
  const std::vector<Jet<1>>& pPsi = S.pPsij;
  double Psi = 0, Psid = 0;
  for (int i = 0; i < n; ++i) { Psi += pPsi[i].c[0] * y[i]; Psid += pPsi[i].c[1] * y[i] + pPsi[i].c[0] * f[i]; }
  const double Phi = y[L.Phi], Phid = f[L.Phi];
  const double Pi = y[L.F(2)] + y[L.G(0)] + y[L.G(2)];
  const double Pid = f[L.F(2)] + f[L.G(0)] + f[L.G(2)];
  const double Pidd = g[L.F(2)] + g[L.G(0)] + g[L.G(2)];
  const double ub = y[L.tb] / k, ubd = f[L.tb] / k;
  const double ST = V * (y[L.F(0)] / 4 + Psi + Pi / 16) + Ek * (Psid + Phid) + (Vd * ub + V * ubd) / k +
                    3.0 / (16.0 * k * k) * (Vdd * Pi + 2 * Vd * Pid + V * Pidd);
  const double chi = B.tau0 - tau;
  const double SE = 3.0 / 16.0 * V * Pi / ((k * chi) * (k * chi));
  const double Spsi = (tau >= B.taurec) ? -(Psi + Phi) * (tau - B.taurec) / (B.tau0 - B.taurec) / (B.tau0 - tau) : 0.0;
  src[0] = k * ST; src[1] = k * k * SE; src[2] = Spsi;
}

void PtSink::emit(int it, double tau, const double* y) {
  const int n = S.n;
  if (mode == 0) {
    double* o = out + (size_t)it * 3;
    if (!y) { o[0] = o[1] = o[2] = 0; return; }
    pt_sources(S, tau, y, o);
  } else if (mode == 2) {
    double* o = out + (size_t)it * n;
    for (int i = 0; i < n; ++i) o[i] = y ? y[i] : 0.0;
  }
}

// total matter gauge-invariant overdensity (src/observables/fourier.jl:39-52, generic_species.jl:48)
static double pt_delta_m(const orc_bg& B, double k, double tau, const double* y) {
  const Cosmo& P = B.P; PtLayout L(P);
  PtCoef<double> C; pt_coef_spline<double>(B, tau, C);
  const double a = C.a, Hc = C.Hc, ia3 = 1 / (a * a * a);
  double rc = P.Oc0 * ia3, rb = P.Ob0 * ia3;
  double num = rc * (y[L.dc] + 3 * Hc * y[L.tc] / (k * k)) + rb * (y[L.db] + 3 * Hc * y[L.tb] / (k * k));
  double den = rc + rb;
  if (P.nx > 0) {
    const double wh = P.Oh0 / P.Irho0 / (a * a * a * a);
    double I0 = 0, I1 = 0, Ir = 0;
    for (int i = 0; i < P.nx; ++i) {
      const double E = std::sqrt(P.xq[i] * P.xq[i] + P.y0 * P.y0 * a * a);
      I0 += P.Wq[i] * E * y[L.H(i, 0)]; I1 += P.Wq[i] * P.xq[i] * y[L.H(i, 1)]; Ir += P.Wq[i] * E;
    }
    num += wh * (I0 + 3 * Hc * I1 / k);
    den += wh * Ir;
  }
  return num / den;
}

}  // namespace orc

extern "C" int orc_pt_nstate(const orc_model* m) {
  return 5 + 2 * (m->lmax_g + 1) + (m->lmax_nu + 1) + m->nx * (m->lmax_h + 1);
}

extern "C" int orc_pt_rhs(const orc_bg* b, double k, double tau, const double* y, double* f, double* J, double* ft) {
  PtSys sys(*b, k);
  sys.rhs(tau, y, f);
  if (J) sys.jac(tau, y, J, ft);
  return 0;
}

extern "C" int orc_pt_initial(const orc_bg* b, double k, double tau, double* y, double* extra) {
  pt_initial(*b, k, tau, y, extra);
  return 0;
}

extern "C" int orc_pt_solve(const orc_bg* b, int nk, const double* ks, const double* tau_ini, int ntau,
                            const double* taus, int mode, double* out, int* status, long* stats) {
  const orc_bg& B = *b;
  const int n = PtLayout(B.P).n;
  const double tstart = B.knots.front().t, tend = B.tau0;
  SparsePattern SP;
  const bool sparse = B.P.pt_linsolve == ORC_LINSOLVE_SPARSE;
  if (sparse) build_sparse_pattern(B, SP);
#pragma omp parallel for schedule(dynamic, 1)
  for (int ik = 0; ik < nk; ++ik) {
    const double k = ks[ik];
    PtSys dense_sys(B, k);
    SparsePtSys* sp = sparse ? new SparsePtSys(B, k, SP) : nullptr;
    PtSys& sys = sp ? *sp : dense_sys;
    double ti = std::min(std::max(tau_ini[ik], tstart), tend);
    std::vector<double> y(n);
    pt_initial(B, k, ti, y.data(), nullptr);
    double* o = nullptr;
    if (mode == 0) o = out + (size_t)ik * ntau * 3;
    else if (mode == 2) o = out + (size_t)ik * ntau * n;
    PtSink sink(sys, ntau, taus, mode, o);
    // output points at the initial time
    while (mode != 1 && sink.next < ntau && taus[sink.next] <= ti) { sink.emit(sink.next, taus[sink.next], taus[sink.next] < ti ? nullptr : y.data()); ++sink.next; }
    long na = 0, nr = 0;
    int st = rosenbrock(B.P.alg_pt, sys, ti, tend, y.data(), B.P.rtol_pt, B.P.atol_pt, B.P.maxiters, &sink, &na, &nr);
    if (mode != 1) while (sink.next < ntau) { sink.emit(sink.next, taus[sink.next], nullptr); ++sink.next; }
    bool finite = true; for (int i = 0; i < n; ++i) finite = finite && std::isfinite(y[i]);
    if (st == 0 && !finite) st = 3;
    if (mode == 1) out[ik] = pt_delta_m(B, k, tend, y.data());
    if (status) status[ik] = st;
    if (stats) { stats[2 * ik] = na; stats[2 * ik + 1] = nr; }
    delete sp;
  }
  return 0;
}
