// Background stage (host, FP64).  See sbz_background.hpp.
//
//   solvebg + a = 1 callback     src/solve.jl:158-203,427-435
//   bg initial conditions        src/models/cosmologies.jl:76 (ℋ = 1/τ), baryons.jl:28,33,156,164
//   background spline            src/utils.jl:118-127
// The ODE is integrated with the Hairer-Wanner RODAS Rosenbrock method (order 4(3), stiffly
// accurate); the reference uses Rodas5P from OrdinaryDiffEqRosenbrock.
#include "sbz_background.hpp"
#include <algorithm>
#include <cmath>
#include <cstring>

namespace sbz {

// ---------------------------------------------------------------------------------------------
// Gauss rule for the measure x² f0(x) dx on (0,∞), f0 = 1/(e^x+1), via u = 1/(1+x/100):
// discretise the u-measure, build the three-term recurrence (Stieltjes), diagonalise the Jacobi
// matrix with cyclic Jacobi rotations (Golub-Welsch).
int momentum_quadrature(int N, double* xs, double* Ws) {
  if (N < 1 || N > 8) return SBZ_ERR_ARG;
  constexpr int NG = 16, NP = 512;
  double gx[NG], gw[NG];
  for (int i = 0; i < NG; ++i) {
    double z = std::cos(phys::PI * (i + 0.75) / (NG + 0.5)), dp = 1;
    for (int it = 0; it < 64; ++it) {
      double p0 = 1, p1 = z;
      for (int j = 2; j <= NG; ++j) { double p2 = ((2 * j - 1) * z * p1 - (j - 1) * p0) / j; p0 = p1; p1 = p2; }
      dp = NG * (z * p1 - p0) / (z * z - 1);
      const double dz = p1 / dp; z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    gx[i] = z; gw[i] = 2 / ((1 - z * z) * dp * dp);
  }
  std::vector<double> u, w;
  u.reserve(NG * NP); w.reserve(NG * NP);
  for (int p = 0; p < NP; ++p)
    for (int i = 0; i < NG; ++i) {
      const double uu = (p + 0.5 + 0.5 * gx[i]) / NP;
      const double x = 100 * (1 - uu) / uu;
      u.push_back(uu);
      w.push_back(0.5 / NP * gw[i] * 100 / (uu * uu) * x * x / (std::exp(x) + 1));
    }
  const size_t M = u.size();
  std::vector<double> q0(M, 0.0), q1(M, 1.0), q2(M);
  double alpha[8], beta[8], prev = 1;
  for (int k = 0; k < N; ++k) {
    double nn = 0, mm = 0;
    for (size_t i = 0; i < M; ++i) { const double t = w[i] * q1[i] * q1[i]; nn += t; mm += t * u[i]; }
    alpha[k] = mm / nn; beta[k] = k ? nn / prev : nn; prev = nn;
    for (size_t i = 0; i < M; ++i) q2[i] = (u[i] - alpha[k]) * q1[i] - (k ? beta[k] * q0[i] : 0.0);
    std::swap(q0, q1); std::swap(q1, q2);
  }
  double A[64] = {0}, V[64] = {0};
  for (int i = 0; i < N; ++i) {
    A[i * N + i] = alpha[i]; V[i * N + i] = 1;
    if (i + 1 < N) A[i * N + i + 1] = A[(i + 1) * N + i] = std::sqrt(beta[i + 1]);
  }
  for (int sweep = 0; sweep < 64; ++sweep) {
    double off = 0;
    for (int i = 0; i < N; ++i) for (int j = i + 1; j < N; ++j) off += A[i * N + j] * A[i * N + j];
    if (off < 1e-32) break;
    for (int p = 0; p < N; ++p)
      for (int q = p + 1; q < N; ++q) {
        const double apq = A[p * N + q];
        if (apq == 0) continue;
        const double th = (A[q * N + q] - A[p * N + p]) / (2 * apq);
        const double t = (th >= 0 ? 1 : -1) / (std::fabs(th) + std::sqrt(th * th + 1));
        const double cs = 1 / std::sqrt(t * t + 1), sn = t * cs;
        for (int r = 0; r < N; ++r) { const double a = A[r * N + p], b = A[r * N + q]; A[r * N + p] = cs * a - sn * b; A[r * N + q] = sn * a + cs * b; }
        for (int r = 0; r < N; ++r) { const double a = A[p * N + r], b = A[q * N + r]; A[p * N + r] = cs * a - sn * b; A[q * N + r] = sn * a + cs * b; }
        for (int r = 0; r < N; ++r) { const double a = V[r * N + p], b = V[r * N + q]; V[r * N + p] = cs * a - sn * b; V[r * N + q] = sn * a + cs * b; }
      }
  }
  std::vector<std::pair<double, double>> xw(N);
  for (int i = 0; i < N; ++i) {
    const double uu = A[i * N + i];
    xw[i] = {100 * (1 - uu) / uu, beta[0] * V[i] * V[i]};
  }
  std::sort(xw.begin(), xw.end());
  for (int i = 0; i < N; ++i) { xs[i] = xw[i].first; Ws[i] = xw[i].second; }
  return SBZ_OK;
}

void cosmo_derive(Cosmo& P, const sbz_params& p, const sbz_model& m) {
  using namespace phys;
  std::memset(&P, 0, sizeof P);
  P.h = p.h; P.Oc0 = p.Omega_c; P.Ob0 = p.Omega_b; P.T0 = p.T0; P.Neff = p.Neff; P.YHe = p.YHe;
  P.As = std::exp(p.ln_As1e10) / 1e10; P.ns = p.ns; P.m_eV = p.m_nu_eV; P.Nnu = p.N_nu;
  P.Hswitch = m.Hswitch; P.Heswitch = m.Heswitch; P.reion = m.reionization; P.nx = m.nx_h;
  P.H0si = H100 * P.h;
  P.Og0 = PI * PI / 15 * std::pow(kB * P.T0, 4) / (std::pow(hbar, 3) * std::pow(c, 5)) * 8 * PI * GN / (3 * P.H0si * P.H0si);
  P.On0 = P.Neff * 7.0 / 8.0 * std::pow(4.0 / 11.0, 4.0 / 3.0) * P.Og0;
  P.Th0 = std::pow(4.0 / 11.0, 1.0 / 3.0) * P.T0;
  if (P.nx > 0) {
    momentum_quadrature(P.nx, P.xq, P.Wq);
    P.y0 = P.m_eV * eV / (kB * P.Th0);
    P.Irho0 = 0;
    for (int i = 0; i < P.nx; ++i) {
      P.Irho0 += P.Wq[i] * std::sqrt(P.xq[i] * P.xq[i] + P.y0 * P.y0);
      P.dlnf[i] = -P.xq[i] / (1 + std::exp(-P.xq[i]));
    }
    P.Oh0 = P.Nnu * 8 * PI / 3 * 2 / (2 * PI * PI) * std::pow(kB * P.Th0, 4) / std::pow(hbar * c, 3) * P.Irho0 /
            (std::pow(P.H0si * c, 2) / GN);
    P.wh = P.Oh0 / P.Irho0;
  }
  P.OL0 = 1 - (P.Og0 + P.On0 + P.Oc0 + P.Ob0 + P.Oh0);
  P.fHe = P.YHe / (mHe / mH * (1 - P.YHe));
  P.kpivot = 0.05 / Mpc / (H100 / c) / P.h;
  auto E = [](double lam) { return hP * (c / lam); };
  P.EH2s1s = E(lamH2s1s);
  P.EHinf2s = E(lamHinf1s) - P.EH2s1s;
  P.EHe2s1s = E(lamHe2s1s);
  P.EHe2p2s = E(lamHe2p1s) - P.EHe2s1s;
  P.EHeinf2s = E(lamHeinf1s) - P.EHe2s1s;
  P.EHetinf2s = E(lamHetinf2s);
  P.EHet2s1s = E(lamHet2s1s);
  P.EHet2p2s = E(lamHet2p1s) - P.EHet2s1s;
  P.fHe2p1s = c / lamHe2p1s;
  P.fHet2p1s = c / lamHet2p1s;
}

// ---------------------------------------------------------------------------------------------
// RODAS tableau (transformed form): (1/(hγ) - J) U_i = f(Y_i) + Σ C_ij U_j / h, Y_i = y + Σ A_ij U_j
namespace rodas {
constexpr double gam = 0.25;
constexpr double A21 = 1.544, A31 = 0.9466785280815826, A32 = 0.2557011698983284;
constexpr double A41 = 3.314825187068521, A42 = 2.896124015972201, A43 = 0.9986419139977817;
constexpr double A51 = 1.221224509226641, A52 = 6.019134481288629, A53 = 12.53708332932087, A54 = -0.6878860361058950;
constexpr double C21 = -5.6688, C31 = -2.430093356833875, C32 = -0.2063599157091915;
constexpr double C41 = -0.1073529058151375, C42 = -9.594562251023355, C43 = -20.47028614809616;
constexpr double C51 = 7.496443313967647, C52 = -10.24680431464352, C53 = -33.99990352819905, C54 = 11.70890893206160;
constexpr double C61 = 8.083246795921522, C62 = -7.981132988064893, C63 = -31.52159432874371, C64 = 16.31930543123136, C65 = -6.058818238834054;
}  // namespace rodas

namespace {

constexpr int NB = 5;

void bg_f(const Cosmo& P, const double* y, double* f) { background_rhs<double>(P, y, f, nullptr); }

void bg_jac(const Cosmo& P, const double* y, double* J) {
  for (int j = 0; j < NB; ++j) {
    Tay<1> yy[NB], ff[NB];
    for (int i = 0; i < NB; ++i) yy[i] = Tay<1>(y[i]);
    yy[j].c[1] = 1;
    background_rhs<Tay<1>>(P, yy, ff, nullptr);
    for (int i = 0; i < NB; ++i) J[i * NB + j] = ff[i].c[1];
  }
}

bool lu5(double* A, int* piv) {
  for (int k = 0; k < NB; ++k) {
    int p = k;
    for (int i = k + 1; i < NB; ++i) if (std::fabs(A[i * NB + k]) > std::fabs(A[p * NB + k])) p = i;
    piv[k] = p;
    if (!(std::fabs(A[p * NB + k]) > 0) || !std::isfinite(A[p * NB + k])) return false;
    if (p != k) for (int j = 0; j < NB; ++j) std::swap(A[k * NB + j], A[p * NB + j]);
    for (int i = k + 1; i < NB; ++i) {
      const double l = A[i * NB + k] / A[k * NB + k];
      A[i * NB + k] = l;
      for (int j = k + 1; j < NB; ++j) A[i * NB + j] -= l * A[k * NB + j];
    }
  }
  return true;
}
void lusolve5(const double* A, const int* piv, double* b) {
  for (int k = 0; k < NB; ++k) if (piv[k] != k) std::swap(b[k], b[piv[k]]);
  for (int i = 0; i < NB; ++i) for (int j = 0; j < i; ++j) b[i] -= A[i * NB + j] * b[j];
  for (int i = NB - 1; i >= 0; --i) { for (int j = i + 1; j < NB; ++j) b[i] -= A[i * NB + j] * b[j]; b[i] /= A[i * NB + i]; }
}

void hermite5(double t0, const double* y0, const double* f0, double t1, const double* y1, const double* f1, double t, double* out) {
  const double h = t1 - t0, s = (t - t0) / h, s2 = s * s, s3 = s2 * s;
  const double h00 = 2 * s3 - 3 * s2 + 1, h10 = s3 - 2 * s2 + s, h01 = -2 * s3 + 3 * s2, h11 = s3 - s2;
  for (int i = 0; i < NB; ++i) out[i] = h00 * y0[i] + h10 * h * f0[i] + h01 * y1[i] + h11 * h * f1[i];
}

}  // namespace

int background_solve(Background& B, const sbz_params& p, const sbz_model& m, const sbz_opts& o) {
  using namespace rodas;
  Cosmo& P = B.P;
  cosmo_derive(P, p, m);
  B.knots.clear();
  B.status = SBZ_OK;
  const double t0 = o.tau_ini, tmax = o.tau_max, rtol = o.bg_rtol, atol = o.bg_atol;
  B.tau_start = t0;
  // a(τ_ini) from ℋ = 1/τ (Newton on τ ℋ(a) - 1, seeded with the radiation solution)
  double y[NB] = {0, 0, 0, 1, 1};
  {
    double orad = P.Og0 + P.On0 + (P.nx > 0 ? P.wh * 7 * std::pow(phys::PI, 4) / 120 : 0);
    double a = std::sqrt(orad) * t0;
    for (int it = 0; it < 100 && std::isfinite(a); ++it) {
      Tay<1> yy[NB] = {Tay<1>::seed(a), Tay<1>(0.0), Tay<1>(0.0), Tay<1>(1.0), Tay<1>(1.0)}, ff[NB];
      BgState<Tay<1>> st;
      background_rhs<Tay<1>>(P, yy, ff, &st);
      const double g = st.Hc.c[0] * t0 - 1, dg = st.Hc.c[1] * t0;
      const double da = -g / dg;
      a += da;
      if (std::fabs(da) <= 1e-15 * std::fabs(a)) break;
    }
    y[0] = a;
  }
  double f0[NB], ft_unused[NB] = {0};
  (void)ft_unused;
  bg_f(P, y, f0);
  for (int i = 0; i < NB; ++i) if (!std::isfinite(y[i]) || !std::isfinite(f0[i])) { B.status = SBZ_NONFINITE; return B.status; }
  {
    BgKnot k; k.t = t0; std::memcpy(k.y, y, sizeof y); std::memcpy(k.s, f0, sizeof f0); B.knots.push_back(k);
  }
  auto rms = [&](const double* v, const double* ref) {
    double s = 0;
    for (int i = 0; i < NB; ++i) { const double sk = atol + std::fabs(ref[i]) * rtol; s += (v[i] / sk) * (v[i] / sk); }
    return std::sqrt(s / NB);
  };
  double h;
  {
    const double d0 = rms(y, y), d1 = rms(f0, y);
    double h0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * d0 / d1;
    h0 = std::min(h0, tmax - t0);
    double Y[NB], F[NB], D[NB];
    for (int i = 0; i < NB; ++i) Y[i] = y[i] + h0 * f0[i];
    bg_f(P, Y, F);
    for (int i = 0; i < NB; ++i) D[i] = (F[i] - f0[i]) / h0;
    const double d2 = rms(D, y), mx = std::max(d1, d2);
    const double h1 = (mx <= 1e-15 || !std::isfinite(mx)) ? std::max(1e-6, 1e-3 * h0) : std::pow(0.01 / mx, 0.2);
    h = std::min(100 * h0, h1);
    if (!std::isfinite(h) || h <= 0) h = 1e-6 * std::max(1.0, t0);
  }
  double t = t0, errold = 1e-4;
  bool rejected = false, nonfinite = false, hit = false;
  double J[NB * NB], W[NB * NB], U[6][NB], Y[NB], F[NB], y1[NB], f1[NB];
  int piv[NB];
  int64_t iters = 0;
  while (t < tmax) {
    if (++iters > o.maxiters) { B.status = SBZ_MAXITERS; return B.status; }
    if (t + 1.01 * h >= tmax) h = tmax - t;
    if (h <= 1e-14 * std::fabs(t)) { B.status = nonfinite ? SBZ_NONFINITE : SBZ_DTMIN; return B.status; }
    bg_jac(P, y, J);
    const double ihg = 1 / (h * gam), ih = 1 / h;
    for (int i = 0; i < NB * NB; ++i) W[i] = -J[i];
    for (int i = 0; i < NB; ++i) W[i * NB + i] += ihg;
    double err = NAN;
    if (lu5(W, piv)) {
      for (int i = 0; i < NB; ++i) U[0][i] = f0[i];
      lusolve5(W, piv, U[0]);
      for (int i = 0; i < NB; ++i) Y[i] = y[i] + A21 * U[0][i];
      bg_f(P, Y, F);
      for (int i = 0; i < NB; ++i) U[1][i] = F[i] + ih * C21 * U[0][i];
      lusolve5(W, piv, U[1]);
      for (int i = 0; i < NB; ++i) Y[i] = y[i] + A31 * U[0][i] + A32 * U[1][i];
      bg_f(P, Y, F);
      for (int i = 0; i < NB; ++i) U[2][i] = F[i] + ih * (C31 * U[0][i] + C32 * U[1][i]);
      lusolve5(W, piv, U[2]);
      for (int i = 0; i < NB; ++i) Y[i] = y[i] + A41 * U[0][i] + A42 * U[1][i] + A43 * U[2][i];
      bg_f(P, Y, F);
      for (int i = 0; i < NB; ++i) U[3][i] = F[i] + ih * (C41 * U[0][i] + C42 * U[1][i] + C43 * U[2][i]);
      lusolve5(W, piv, U[3]);
      for (int i = 0; i < NB; ++i) Y[i] = y[i] + A51 * U[0][i] + A52 * U[1][i] + A53 * U[2][i] + A54 * U[3][i];
      bg_f(P, Y, F);
      for (int i = 0; i < NB; ++i) U[4][i] = F[i] + ih * (C51 * U[0][i] + C52 * U[1][i] + C53 * U[2][i] + C54 * U[3][i]);
      lusolve5(W, piv, U[4]);
      for (int i = 0; i < NB; ++i) Y[i] += U[4][i];
      bg_f(P, Y, F);
      for (int i = 0; i < NB; ++i) U[5][i] = F[i] + ih * (C61 * U[0][i] + C62 * U[1][i] + C63 * U[2][i] + C64 * U[3][i] + C65 * U[4][i]);
      lusolve5(W, piv, U[5]);
      double s = 0;
      for (int i = 0; i < NB; ++i) {
        y1[i] = Y[i] + U[5][i];
        const double sk = atol + rtol * std::max(std::fabs(y[i]), std::fabs(y1[i]));
        s += (U[5][i] / sk) * (U[5][i] / sk);
      }
      err = std::sqrt(s / NB);
    }
    if (std::isfinite(err) && err <= 1) {
      const double tn = (h == tmax - t) ? tmax : t + h;
      bg_f(P, y1, f1);
      if (y1[0] >= 1.0) {  // a = 1 inside this step: bisect the step's Hermite interpolant
        double lo = t, hi = tn, tmp[NB];
        for (int it = 0; it < 200; ++it) {
          const double mid = 0.5 * (lo + hi);
          if (mid <= lo || mid >= hi) break;
          hermite5(t, y, f0, tn, y1, f1, mid, tmp);
          (tmp[0] >= 1.0 ? hi : lo) = mid;
        }
        BgKnot k; k.t = hi;
        hermite5(t, y, f0, tn, y1, f1, hi, k.y);
        bg_f(P, k.y, k.s);
        B.knots.push_back(k);
        hit = true;
        break;
      }
      t = tn;
      std::memcpy(y, y1, sizeof y);
      std::memcpy(f0, f1, sizeof f0);
      BgKnot k; k.t = t; std::memcpy(k.y, y, sizeof y); std::memcpy(k.s, f0, sizeof f0); B.knots.push_back(k);
      double fac = 0.9 * std::pow(std::max(err, 1e-10), -0.175) * std::pow(errold, 0.1);
      fac = std::min(10.0, std::max(0.2, fac));
      if (rejected) fac = std::min(fac, 1.0);
      errold = std::max(err, 1e-4);
      h *= fac;
      rejected = false; nonfinite = false;
    } else {
      rejected = true;
      if (!std::isfinite(err)) { nonfinite = true; h *= 0.2; }
      else h *= std::max(0.2, 0.9 * std::pow(err, -0.25));
    }
  }
  if (!hit) { B.status = SBZ_NONFINITE; return B.status; }
  B.tau0 = B.knots.back().t;
  B.kappa0 = B.knots.back().y[1];
  // smooth spline slopes for the stiff unknowns ΔT, XH⁺, XHe⁺: derivative of the interpolating
  // polynomial through the 5 nearest knots (their ODE right-hand sides amplify rounding-level
  // departures from quasi-equilibrium by the enormous rates)
  {
    const int nk = (int)B.knots.size();
    std::vector<double> sl((size_t)3 * nk);
    // the stencils skip knot 0 (the off-equilibrium initial condition ΔT = 0 and the ~1e-14-wide
    // transient after it must not leak into the slopes)
    for (int i = 0; i < nk; ++i) {
      const int lo = std::max(1, std::min(i - 2, nk - 5)), hi = std::min(nk - 1, lo + 4);
      const double xi = B.knots[i].t;
      double d[3] = {0, 0, 0};
      for (int j = lo; j <= hi; ++j) {
        const double xj = B.knots[j].t;
        double wgt;
        if (j == i) { wgt = 0; for (int q = lo; q <= hi; ++q) if (q != i) wgt += 1 / (xi - B.knots[q].t); }
        else {
          double num = 1, den = 1;
          for (int q = lo; q <= hi; ++q) { if (q == j) continue; den *= xj - B.knots[q].t; if (q != i) num *= xi - B.knots[q].t; }
          wgt = num / den;
        }
        for (int c = 0; c < 3; ++c) d[c] += wgt * B.knots[j].y[2 + c];
      }
      for (int c = 0; c < 3; ++c) sl[3 * i + c] = d[c];
    }
    for (int i = 0; i < nk; ++i) for (int c = 0; c < 3; ++c) B.knots[i].s[2 + c] = sl[3 * i + c];
  }
  // recombination time: maximum of the visibility (golden section around the best knot)
  auto vis = [&](double tau) {
    double yy[NB], ff[NB];
    background_spline(B, tau, yy);
    bg_f(P, yy, ff);
    return -ff[1] * std::exp(-(yy[1] - B.kappa0));
  };
  int imax = 0; double vmax = -1;
  for (size_t i = 0; i < B.knots.size(); ++i) { const double v = vis(B.knots[i].t); if (v > vmax) { vmax = v; imax = (int)i; } }
  double lo = B.knots[std::max(imax - 1, 0)].t, hi = B.knots[std::min<size_t>(imax + 1, B.knots.size() - 1)].t;
  const double gr = 0.5 * (std::sqrt(5.0) - 1);
  double x1 = hi - gr * (hi - lo), x2 = lo + gr * (hi - lo), v1 = vis(x1), v2 = vis(x2);
  for (int it = 0; it < 200 && hi - lo > 1e-15 * hi; ++it) {
    if (v1 > v2) { hi = x2; x2 = x1; v2 = v1; x1 = hi - gr * (hi - lo); v1 = vis(x1); }
    else { lo = x1; x1 = x2; v1 = v2; x2 = lo + gr * (hi - lo); v2 = vis(x2); }
  }
  B.taurec = 0.5 * (lo + hi);
  return B.status;
}

// Hermite spline of the unknowns; S = double (value) or Tay<1> (value and d/dτ)
template <class S>
static void spline_at(const Background& B, double tau, S* y) { knots_spline<S>(B.knots.data(), (int)B.knots.size(), tau, y); }

void background_spline(const Background& B, double tau, double* y) { spline_at<double>(B, tau, y); }

void background_eval(const Background& B, double tau, double* out) {
  Tay<1> y[NB], f[NB];
  spline_at<Tay<1>>(B, tau, y);
  BgState<Tay<1>> st;
  background_rhs<Tay<1>>(B.P, y, f, &st);
  const double kap = y[1].c[0] - B.kappa0;
  const double ek = std::exp(-kap);
  // Taylor-mode κ̈ at the splined state for v̇
  Tay<2> z[NB], g[NB];
  double yv[NB]; background_spline(B, tau, yv);
  for (int j = 0; j < NB; ++j) z[j] = Tay<2>(yv[j]);
  for (int ord = 0; ord < 2; ++ord) {
    background_rhs<Tay<2>>(B.P, z, g, nullptr);
    for (int j = 0; j < NB; ++j) z[j].c[ord + 1] = g[j].c[ord] / (ord + 1);
  }
  background_rhs<Tay<2>>(B.P, z, g, nullptr);
  const double kd = g[1].c[0], kdd = g[1].c[1];
  const double r[9] = {st.a.c[0], st.Hc.c[0], st.kd.c[0], kap, -kd * ek, (kd * kd - kdd) * ek, st.cs2.c[0], st.Xe.c[0], st.Tb.c[0]};
  std::memcpy(out, r, sizeof r);
}

// Coefficient table on ln τ nodes (see kTabStride)
void background_table_grid(Background& B, int ntab) {
  B.ntab = ntab;
  B.lnt0 = std::log(B.tau_start);
  B.dlnt = (std::log(B.tau0) - B.lnt0) / (ntab - 1);
  B.tab.clear();
  B.tabtau.resize(ntab);
  for (int g = 0; g < ntab; ++g)
    B.tabtau[g] = (g == ntab - 1) ? B.tau0 : (g == 0 ? B.tau_start : std::exp(B.lnt0 + g * B.dlnt));
}

void background_table_values(Background& B) {
  const int ntab = B.ntab;
  B.tab.assign((size_t)ntab * kTabStride, 0.0);
  // nodes are independent; inside an outer parallel loop over cosmologies this runs serially
#pragma omp parallel for schedule(static)
  for (int g = 0; g < ntab; ++g) table_node(B.P, B.knots.data(), (int)B.knots.size(), B.kappa0, B.tabtau[g], &B.tab[(size_t)g * kTabStride]);
}

void table_eval(const Background& B, double tau, double* out) {
  int g = (int)std::floor((std::log(tau) - B.lnt0) / B.dlnt);
  g = std::max(0, std::min(g, B.ntab - 2));
  if (tau < B.tabtau[g] && g > 0) --g;
  else if (tau > B.tabtau[g + 1] && g < B.ntab - 2) ++g;
  const double t0 = B.tabtau[g], h = B.tabtau[g + 1] - t0, s = (tau - t0) / h, s2 = s * s, s3 = s2 * s;
  const double* A = &B.tab[(size_t)g * kTabStride];
  const double* C = &B.tab[(size_t)(g + 1) * kTabStride];
  for (int q = 0; q < 7; ++q)
    out[q] = (2 * s3 - 3 * s2 + 1) * A[2 * q] + (s3 - 2 * s2 + s) * h * A[2 * q + 1] + (3 * s2 - 2 * s3) * C[2 * q] + (s3 - s2) * h * C[2 * q + 1];
}

}  // namespace sbz
