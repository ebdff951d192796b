// One node of the per-cosmology background coefficient table, shared by the host build
// (sbz_background.cpp) and the device build (sbz_table.cu), so both evaluate the same arithmetic.
//
// A node at time τ holds (value, d/dτ) pairs of a, ℋ, κ̇, c_s² — the chain rule through the
// cubic Hermite spline of the background unknowns — and of e^{-κ}, κ̈, κ⃛ — a Taylor-mode
// expansion of the background ODE at the splined state (the line-of-sight sources differentiate
// the background along its ODE, src/models/cosmologies.jl:99-105).
#pragma once
#include "sbz_jet.cuh"
#include "sbz_physics.cuh"

namespace sbz {

constexpr int kBgUnknowns = 5;
constexpr int kTabValues = 14;  // doubles per node: seven (value, d/dτ) pairs

struct BgKnot { double t, y[kBgUnknowns], s[kBgUnknowns]; };  // time, unknowns, spline slopes

// Hermite spline of the unknowns at τ from nk knots; S = double (value) or Tay<1> (value, d/dτ).
template <class S>
SBZ_HD void knots_spline(const BgKnot* K, int nk, double tau, S* y) {
  int lo = 0, hi = nk - 1;
  if (tau <= K[0].t) hi = 1;
  else if (tau >= K[hi].t) lo = hi - 1;
  else while (hi - lo > 1) { const int mid = (lo + hi) >> 1; (K[mid].t <= tau ? lo : hi) = mid; }
  const BgKnot &A = K[lo], &Bk = K[lo + 1];
  const double h = Bk.t - A.t, s = (tau - A.t) / h, s2 = s * s, s3 = s2 * s;
  const double h00 = 2 * s3 - 3 * s2 + 1, h10 = s3 - 2 * s2 + s, h01 = -2 * s3 + 3 * s2, h11 = s3 - s2;
  const double g00 = (6 * s2 - 6 * s) / h, g10 = 3 * s2 - 4 * s + 1, g01 = (6 * s - 6 * s2) / h, g11 = 3 * s2 - 2 * s;
  for (int j = 0; j < kBgUnknowns; ++j) {
    y[j] = S(h00 * A.y[j] + h10 * h * A.s[j] + h01 * Bk.y[j] + h11 * h * Bk.s[j]);
    if constexpr (sizeof(S) > sizeof(double)) y[j].c[1] = g00 * A.y[j] + g10 * A.s[j] + g01 * Bk.y[j] + g11 * Bk.s[j];
  }
}

// The kTabValues doubles of the node at τ.
SBZ_HD void table_node(const Cosmo& P, const BgKnot* K, int nk, double kappa0, double tau, double* T) {
  {  // chain rule through the spline: the perturbation right-hand-side coefficients
    Tay<1> y[kBgUnknowns], f[kBgUnknowns];
    knots_spline<Tay<1>>(K, nk, tau, y);
    BgState<Tay<1>> st;
    background_rhs<Tay<1>>(P, y, f, &st);
    T[0] = st.a.c[0]; T[1] = st.a.c[1];
    T[2] = st.Hc.c[0]; T[3] = st.Hc.c[1];
    T[4] = st.kd.c[0]; T[5] = st.kd.c[1];
    T[6] = st.cs2.c[0]; T[7] = st.cs2.c[1];
  }
  {  // Taylor mode through the splined state: visibility derivatives for the sources
    constexpr int N = 4;
    double yv[kBgUnknowns];
    knots_spline<double>(K, nk, tau, yv);
    Tay<N> z[kBgUnknowns], g[kBgUnknowns];
    for (int j = 0; j < kBgUnknowns; ++j) z[j] = Tay<N>(yv[j]);
    for (int ord = 0; ord < N; ++ord) {
      background_rhs<Tay<N>>(P, z, g, nullptr);
      for (int j = 0; j < kBgUnknowns; ++j) z[j].c[ord + 1] = g[j].c[ord] / (ord + 1);
    }
    background_rhs<Tay<N>>(P, z, g, nullptr);
    const Tay<N> ek = exp(-(z[1] - kappa0));
    T[8] = ek.c[0]; T[9] = ek.c[1];
    T[10] = g[1].c[1]; T[11] = 2 * g[1].c[2];
    T[12] = 2 * g[1].c[2]; T[13] = 6 * g[1].c[3];
  }
}

}  // namespace sbz
