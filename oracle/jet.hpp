// Truncated Taylor-series arithmetic for the CPU oracle (test infrastructure only).
//
// Jet<N> holds the normalised Taylor coefficients c[0..N] of a function of conformal time,
// f(tau + s) = sum_k c[k] s^k.  Jet<1> is a forward-mode dual number.  The oracle uses it
//   * to differentiate the background right-hand side (Jacobian of the background stage),
//   * for the explicit time derivative df/dtau of the perturbation stage (the reference gets
//     the same quantity from forward-mode AD through its background spline, src/solve.jl:204,227),
//   * for Taylor-mode expansions of the background trajectory, which give the exact
//     higher derivatives (kappa'', kappa''') that the reference's symbolic expansion of the
//     line-of-sight sources produces (src/models/cosmologies.jl:99-105).
#pragma once
#include <cmath>

namespace orc {

template <int N>
struct Jet {
  double c[N + 1];
  Jet() { for (int i = 0; i <= N; ++i) c[i] = 0.0; }
  Jet(double v) { c[0] = v; for (int i = 1; i <= N; ++i) c[i] = 0.0; }
  static Jet var(double v) { Jet r(v); if (N >= 1) r.c[1] = 1.0; return r; }
  double val() const { return c[0]; }
};

template <class T> inline double value_of(const T& x) { return x.c[0]; }
inline double value_of(double x) { return x; }

template <int N> inline Jet<N> operator+(const Jet<N>& a, const Jet<N>& b) { Jet<N> r; for (int i = 0; i <= N; ++i) r.c[i] = a.c[i] + b.c[i]; return r; }
template <int N> inline Jet<N> operator-(const Jet<N>& a, const Jet<N>& b) { Jet<N> r; for (int i = 0; i <= N; ++i) r.c[i] = a.c[i] - b.c[i]; return r; }
template <int N> inline Jet<N> operator-(const Jet<N>& a) { Jet<N> r; for (int i = 0; i <= N; ++i) r.c[i] = -a.c[i]; return r; }
template <int N> inline Jet<N> operator+(const Jet<N>& a, double b) { Jet<N> r = a; r.c[0] += b; return r; }
template <int N> inline Jet<N> operator+(double b, const Jet<N>& a) { return a + b; }
template <int N> inline Jet<N> operator-(const Jet<N>& a, double b) { Jet<N> r = a; r.c[0] -= b; return r; }
template <int N> inline Jet<N> operator-(double b, const Jet<N>& a) { Jet<N> r = -a; r.c[0] += b; return r; }
template <int N> inline Jet<N> operator*(const Jet<N>& a, double b) { Jet<N> r; for (int i = 0; i <= N; ++i) r.c[i] = a.c[i] * b; return r; }
template <int N> inline Jet<N> operator*(double b, const Jet<N>& a) { return a * b; }
template <int N> inline Jet<N> operator/(const Jet<N>& a, double b) { return a * (1.0 / b); }
template <int N> inline Jet<N> operator*(const Jet<N>& a, const Jet<N>& b) {
  Jet<N> r;
  for (int k = 0; k <= N; ++k) { double s = 0; for (int j = 0; j <= k; ++j) s += a.c[j] * b.c[k - j]; r.c[k] = s; }
  return r;
}
template <int N> inline Jet<N> operator/(const Jet<N>& a, const Jet<N>& b) {
  Jet<N> r;
  for (int k = 0; k <= N; ++k) { double s = a.c[k]; for (int j = 1; j <= k; ++j) s -= b.c[j] * r.c[k - j]; r.c[k] = s / b.c[0]; }
  return r;
}
template <int N> inline Jet<N> operator/(double a, const Jet<N>& b) { return Jet<N>(a) / b; }
template <int N> inline Jet<N>& operator+=(Jet<N>& a, const Jet<N>& b) { a = a + b; return a; }
template <int N> inline Jet<N>& operator-=(Jet<N>& a, const Jet<N>& b) { a = a - b; return a; }
template <int N> inline Jet<N>& operator*=(Jet<N>& a, const Jet<N>& b) { a = a * b; return a; }
template <int N> inline Jet<N>& operator+=(Jet<N>& a, double b) { a.c[0] += b; return a; }
template <int N> inline Jet<N>& operator-=(Jet<N>& a, double b) { a.c[0] -= b; return a; }

template <int N> inline Jet<N> exp(const Jet<N>& u) {
  Jet<N> w; w.c[0] = std::exp(u.c[0]);
  for (int k = 1; k <= N; ++k) { double s = 0; for (int j = 1; j <= k; ++j) s += j * u.c[j] * w.c[k - j]; w.c[k] = s / k; }
  return w;
}
template <int N> inline Jet<N> log(const Jet<N>& u) {
  Jet<N> w; w.c[0] = std::log(u.c[0]);
  for (int k = 1; k <= N; ++k) { double s = 0; for (int j = 1; j < k; ++j) s += j * w.c[j] * u.c[k - j]; w.c[k] = (u.c[k] - s / k) / u.c[0]; }
  return w;
}
// u^p for a constant exponent p (u0 > 0): k u0 w_k = sum_{j<k} (p(k-j) - j) u_{k-j} w_j
template <int N> inline Jet<N> pow(const Jet<N>& u, double p) {
  Jet<N> w; w.c[0] = std::pow(u.c[0], p);
  for (int k = 1; k <= N; ++k) { double s = 0; for (int j = 0; j < k; ++j) s += (p * (k - j) - j) * u.c[k - j] * w.c[j]; w.c[k] = s / (k * u.c[0]); }
  return w;
}
template <int N> inline Jet<N> sqrt(const Jet<N>& u) { return pow(u, 0.5); }
template <int N> inline Jet<N> tanh(const Jet<N>& u) {
  Jet<N> t, s; t.c[0] = std::tanh(u.c[0]); s.c[0] = 1.0 - t.c[0] * t.c[0];
  for (int k = 1; k <= N; ++k) {
    double a = 0; for (int j = 1; j <= k; ++j) a += j * u.c[j] * s.c[k - j]; t.c[k] = a / k;
    double b = 0; for (int j = 0; j <= k; ++j) b += t.c[j] * t.c[k - j]; s.c[k] = -b;
  }
  return t;
}

// Plain-double overloads so the same templates run with T = double.
using std::exp; using std::log; using std::pow; using std::sqrt; using std::tanh;

}  // namespace orc
