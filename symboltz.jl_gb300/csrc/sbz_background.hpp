// Background stage on the host: derived parameters, momentum quadrature, the background ODE
// solve to a = 1, its cubic Hermite spline, and the per-cosmology coefficient table that the
// perturbation kernels read from HBM.
#pragma once
#include <vector>
#include "sbz_physics.cuh"
#include "sbz_table.cuh"
#include "../../include/symboltz_gb300.h"

namespace sbz {

// Number of doubles per table node: (value, d/dτ) pairs of
//   a, ℋ, κ̇, c_s² (chain rule through the background spline), e^{-κ}, κ̈, κ⃛ (Taylor mode).
constexpr int kTabStride = kTabValues;

struct Background {
  Cosmo P;
  int status = 0;
  double tau_start = 0, tau0 = 0, kappa0 = 0, taurec = 0;
  std::vector<BgKnot> knots;
  // coefficient table: ln τ uniform on [ln tau_start, ln tau0]
  int ntab = 0;
  double lnt0 = 0, dlnt = 0;
  std::vector<double> tab;     // ntab * kTabStride; empty until background_table_values
  std::vector<double> tabtau;  // ntab node times
};

int momentum_quadrature(int N, double* x, double* W);
void cosmo_derive(Cosmo& P, const sbz_params& p, const sbz_model& m);
// Solves one cosmology; returns 0 on success or an SBZ_* status code.
int background_solve(Background& B, const sbz_params& p, const sbz_model& m, const sbz_opts& o);
// Node times of the coefficient table (cheap); the values are built by background_table_values on
// the host or by the device kernel (sbz_table.cu) from the knots.
void background_table_grid(Background& B, int ntab);
void background_table_values(Background& B);
inline void background_table(Background& B, int ntab) { background_table_grid(B, ntab); background_table_values(B); }
// Spline of the unknowns at τ (value only)
void background_spline(const Background& B, double tau, double* y);
// Derived quantities at τ: a, ℋ, κ̇, κ, v, v̇, c_s², Xe, Tb (from the spline)
void background_eval(const Background& B, double tau, double* out);
// Hermite interpolation of the coefficient table as the kernels do it: a, ℋ, κ̇, c_s², e^{-κ}, κ̈, κ⃛
void table_eval(const Background& B, double tau, double* out7);

}  // namespace sbz
