// Background physics of the ΛCDM(+massive ν) model, host/device templates.
//
// Follows the reference's component equations:
//   constants                     src/constants.jl:3-50 (CODATA 2018, IAU parsec, atomic masses)
//   Friedmann equation            src/models/gravity.jl:31
//   species densities             src/models/generic_species.jl:30-32, photons.jl:44-46,
//                                 neutrinos.jl:78-86,109-118, cosmologies.jl:78-84,221-227
//   baryon thermodynamics         src/models/baryons.jl:145-212
//   RECFAST 1.5.2 recombination   src/models/baryons.jl:14-116 (Hswitch 0/1, Heswitch 0/6)
//   tanh reionization             src/models/baryons.jl:128-138,201-205
// The background unknowns are y = [a, κ̃ (optical depth from the start), ΔT = Tb - Tγ, XH⁺, XHe⁺].
#pragma once
#include "sbz_jet.cuh"

namespace sbz {

namespace phys {
constexpr double PI = 3.14159265358979323846;
constexpr double c = 299792458.0;
constexpr double hP = 6.62607015e-34;
constexpr double hbar = hP / (2 * PI);
constexpr double kB = 1.380649e-23;
constexpr double GN = 6.67430e-11;
constexpr double sigmaSB = 5.670374419e-8;
constexpr double aR = 4.0 / c * sigmaSB;
constexpr double sigmaT = 6.6524587321e-29;
constexpr double me = 9.1093837015e-31;
constexpr double amu = 1.66053906660e-27;
constexpr double mH = 1.008 * amu;
constexpr double mHe = 4.0026022 * amu;
constexpr double Mpc = 1e6 * 3.0856775814913673e16;
constexpr double H100 = 1e5 / Mpc;
constexpr double eV = 1.602176634e-19;
// atomic transitions (wavelengths in m); energies E = h (c / λ)
constexpr double lamH2s1s = 121.56700e-9, lamHinf1s = 91.17534e-9;
constexpr double lamHeinf1s = 50.42590e-9, lamHe2s1s = 60.14045e-9, lamHe2p1s = 58.43344e-9;
constexpr double lamHetinf2s = 260.0463e-9, lamHet2p1s = 59.1411e-9, lamHet2s1s = 62.5563e-9;
constexpr double EHepinf1s = 54.4178 * eV;
}  // namespace phys

// Everything the background needs for one cosmology (plain data; copied to the device).
struct Cosmo {
  // inputs
  double h, Oc0, Ob0, T0, Neff, YHe, As, ns, m_eV, Nnu;
  int Hswitch, Heswitch, reion, nx;
  // derived
  double H0si;        // H0 in 1/s
  double Og0, On0, Oh0, OL0;
  double fHe, kpivot, Th0, y0, Irho0, wh;  // wh = Oh0/Irho0
  double xq[8], Wq[8], dlnf[8];
  // transition energies (J)
  double EHinf2s, EH2s1s, EHeinf2s, EHe2s1s, EHe2p2s, EHetinf2s, EHet2s1s, EHet2p2s;
  double fHe2p1s, fHet2p1s;
};

template <class S>
SBZ_HD S smooth_step(const S& x, const S& v1, const S& v2, double k) {  // src/utils.jl:37
  return 0.5 * ((v1 + v2) + (v2 - v1) * tanh(k * x));
}

// Derived background quantities returned alongside the RHS.
template <class S> struct BgState { S a, Hc, kd, Xe, Tb, cs2; };

// dy/dτ of the background unknowns (τ in 1/H0).  Templated on the scalar so the same code gives
// values (double), the Jacobian (Tay<1>) and Taylor expansions (Tay<N>).
template <class S>
SBZ_HD void background_rhs(const Cosmo& P, const S* y, S* dy, BgState<S>* st) {
  using namespace phys;
  const S a = y[0];
  const S ia = 1.0 / a;
  const S ia3 = ia * ia * ia;
  const S ia4 = ia3 * ia;
  S Omega = (P.Og0 + P.On0) * ia4 + (P.Oc0 + P.Ob0) * ia3 + S(P.OL0);
  if (P.nx > 0) {
    S Ir(0.0);
    const S ya2 = (P.y0 * P.y0) * (a * a);
    for (int i = 0; i < P.nx; ++i) Ir += P.Wq[i] * sqrt(P.xq[i] * P.xq[i] + ya2);
    Omega += P.wh * Ir * ia4;
  }
  const S adot = sqrt(Omega) * (a * a);
  const S Hc = adot * ia;
  const S Hsi = (P.H0si * ia) * Hc;
  const S Tg = P.T0 * ia;
  const S Tb = y[2] + Tg;
  const S XH = y[3], XHe = y[4];
  const S nH = ((1 - P.YHe) * 3 / (8 * PI) * P.Ob0 * P.H0si * P.H0si / GN / mH) * ia3;
  const S nHe = P.fHe * nH;
  const S beta = 1.0 / (kB * Tb);
  const S lam = hP / sqrt((2 * PI * me * kB) * Tb);
  const S lam3 = lam * lam * lam;
  // doubly ionised helium in Saha equilibrium
  const S RHep = exp(-beta * EHepinf1s) / (nH * lam3);
  const S g = 1 + P.fHe + RHep;
  const S XHepp = 2 * RHep * P.fHe / g / (1 + sqrt(1 + 4 * RHep * P.fHe / (g * g)));
  S Xe = XH + P.fHe * XHe + XHepp;
  if (P.reion) {
    // (1+z)^n tanh steps: z = 7.6711, Δz = 0.5, n = 3/2 (H + He⁺) and z = 3.5, Δz = 0.5, n = 1 (He⁺⁺)
    const double k1 = 1.0 / (1.5 * ::sqrt(1 + 7.6711) * 0.5);
    Xe += smooth_step(::pow(1 + 7.6711, 1.5) - pow(ia, 1.5), S(0.0), S(1 + P.fHe), k1);
    Xe += smooth_step((1 + 3.5) - ia, S(0.0), S(P.fHe), 1.0 / 0.5);
  }
  const S ne = Xe * nH;
  const S conv = a * (1.0 / P.H0si);
  const S kd = -(sigmaT * c) * conv * ne;
  const S Tg2 = Tg * Tg;
  const S DT = -2 * Tb * Hc - ((8.0 / 3.0) * sigmaT * aR / (me * c)) * conv * (Tg2 * Tg2) * Xe / (1 + P.fHe + Xe) * y[2];
  dy[0] = adot;
  dy[1] = kd;
  dy[2] = DT + Tg * Hc;
  // hydrogen: effective three-level atom with fudge factor and Gaussian K correction
  const double FH = (P.Hswitch == 0) ? 1.14 : 1.125;
  const S t4 = Tb * 1e-4;
  const S alphaH = (FH * 1e-19 * 4.309) * pow(t4, -0.6166) / (1 + 0.6703 * pow(t4, 0.5300));
  const S betaH = alphaH / lam3 * exp(-beta * P.EHinf2s);
  S Kfit(1.0);
  if (P.Hswitch == 1) {
    const S la = log(a);
    const S u1 = (la + 7.28) * (1 / 0.18), u2 = (la + 6.73) * (1 / 0.33);
    Kfit = 1 - 0.14 * exp(-(u1 * u1)) + 0.079 * exp(-(u2 * u2));
  }
  const double LamH = 8.2245809, LamHe = 51.3;
  const S KH = Kfit * (lamH2s1s * lamH2s1s * lamH2s1s / (8 * PI)) / Hsi;
  const S omXH = 1 - XH;
  const S CH = smooth_step(XH - 0.99, (1 + KH * LamH * nH * omXH) / (1 + KH * (LamH + betaH) * nH * omXH), S(1.0), 1e3);
  dy[3] = -conv * CH * (alphaH * XH * ne - betaH * omXH * exp(-beta * P.EH2s1s));
  // helium: singlet (+ triplet and line-escape corrections for Heswitch = 6)
  const S sq2 = sqrt(Tb * (1.0 / 3.0)), sq1 = sqrt(Tb * ::pow(10.0, -5.114));
  const S alphaHe = ::pow(10.0, -16.744) / (sq2 * pow(1 + sq2, 1 - 0.711) * pow(1 + sq1, 1 + 0.711));
  const S betaHe = 4 * alphaHe / lam3 * exp(-beta * P.EHeinf2s);
  const S iK0 = (8 * PI / (lamHe2p1s * lamHe2p1s * lamHe2p1s)) * Hsi;
  const S omXHe = 1 - XHe;
  const double eps = 1e-9;
  S iKsum = iK0;
  S dXHet(0.0);
  if (P.Heswitch == 6) {
    const double A2ps = 1.798287e9, A2pt = 177.58;
    const S common = 3 * P.fHe * (omXHe + eps) * (c * c) / (8 * PI * sqrt(2 * PI / (beta * (mHe * c * c))) * (omXH + eps));
    const S tauHe = 3 * A2ps * nHe * (omXHe + eps) / iK0;
    iKsum = iKsum - exp(-tauHe) * iK0;
    const S g2ps = common * (A2ps / (1.436289e-22 * P.fHe2p1s * P.fHe2p1s * P.fHe2p1s));
    iKsum = iKsum + A2ps / (1 + 0.36 * pow(g2ps, 0.86)) * 3 * nHe * omXHe;
    const S alphaHet = ::pow(10.0, -16.306) / (sq2 * pow(1 + sq2, 1 - 0.761) * pow(1 + sq1, 1 + 0.761));
    const S betaHet = (4.0 / 3.0) * alphaHet / lam3 * exp(-beta * P.EHetinf2s);
    const S tauHet = (A2pt * 3 * lamHet2p1s * lamHet2p1s * lamHet2p1s / (8 * PI)) * nHe * (omXHe + eps) / Hsi;
    const S pHet = (1 - exp(-tauHet)) / tauHet;
    const S g2pt = common * (A2pt / (1.484872e-22 * P.fHet2p1s * P.fHet2p1s * P.fHet2p1s));
    const S CHetnum = A2pt * (pHet + 1 / (1 + 0.66 * pow(g2pt, 0.9)) / 3) * exp(-beta * P.EHet2p2s);
    const S CHet = (eps + CHetnum) / (eps + CHetnum + betaHet);
    dXHet = -conv * CHet * (alphaHet * XHe * ne - betaHet * omXHe * 3 * exp(-beta * P.EHet2s1s));
  }
  const S KHe = 1 / iKsum;
  const S e22 = exp(-beta * P.EHe2p2s);
  const S CHe = smooth_step(XHe - 0.99, (e22 + KHe * LamHe * nHe * omXHe) / (e22 + KHe * (LamHe + betaHe) * nHe * omXHe), S(1.0), 1e3);
  dy[4] = dXHet - conv * CHe * (alphaHe * XHe * ne - betaHe * omXHe * exp(-beta * P.EHe2s1s));
  if (st) {
    st->a = a; st->Hc = Hc; st->kd = kd; st->Xe = Xe; st->Tb = Tb;
    const S muc2 = (mH * c * c) / (1 + (mH / mHe - 1) * P.YHe + Xe * (1 - P.YHe));
    st->cs2 = (kB / muc2) * (Tb - DT / (3 * Hc));
  }
}

}  // namespace sbz
