// Truncated Taylor arithmetic usable on host and device.
//
// sbz::Tay<N> carries f(t+s) = sum_k c[k] s^k.  Tay<1> is a forward-mode dual number (used for
// the background Jacobian and for d/dtau of tabulated coefficients); higher orders give the
// Taylor-mode expansion of the background trajectory needed by the line-of-sight sources
// (kappa'' and kappa''' enter the visibility derivatives, src/models/cosmologies.jl:99-105).
#pragma once
#include <cmath>

#if defined(__CUDACC__)
#define SBZ_HD __host__ __device__ __forceinline__
#else
#define SBZ_HD inline
#endif

namespace sbz {

template <int N>
struct Tay {
  double c[N + 1];
  SBZ_HD Tay() {
#pragma unroll
    for (int i = 0; i <= N; ++i) c[i] = 0.0;
  }
  SBZ_HD Tay(double v) {
    c[0] = v;
#pragma unroll
    for (int i = 1; i <= N; ++i) c[i] = 0.0;
  }
  SBZ_HD static Tay seed(double v) { Tay r(v); if (N >= 1) r.c[1] = 1.0; return r; }
};

#define SBZ_TAY_LOOP _Pragma("unroll") for (int i = 0; i <= N; ++i)
template <int N> SBZ_HD Tay<N> operator+(const Tay<N>& a, const Tay<N>& b) { Tay<N> r; SBZ_TAY_LOOP r.c[i] = a.c[i] + b.c[i]; return r; }
template <int N> SBZ_HD Tay<N> operator-(const Tay<N>& a, const Tay<N>& b) { Tay<N> r; SBZ_TAY_LOOP r.c[i] = a.c[i] - b.c[i]; return r; }
template <int N> SBZ_HD Tay<N> operator-(const Tay<N>& a) { Tay<N> r; SBZ_TAY_LOOP r.c[i] = -a.c[i]; return r; }
template <int N> SBZ_HD Tay<N> operator+(const Tay<N>& a, double b) { Tay<N> r = a; r.c[0] += b; return r; }
template <int N> SBZ_HD Tay<N> operator+(double b, const Tay<N>& a) { Tay<N> r = a; r.c[0] += b; return r; }
template <int N> SBZ_HD Tay<N> operator-(const Tay<N>& a, double b) { Tay<N> r = a; r.c[0] -= b; return r; }
template <int N> SBZ_HD Tay<N> operator-(double b, const Tay<N>& a) { Tay<N> r = -a; r.c[0] += b; return r; }
template <int N> SBZ_HD Tay<N> operator*(const Tay<N>& a, double b) { Tay<N> r; SBZ_TAY_LOOP r.c[i] = a.c[i] * b; return r; }
template <int N> SBZ_HD Tay<N> operator*(double b, const Tay<N>& a) { Tay<N> r; SBZ_TAY_LOOP r.c[i] = a.c[i] * b; return r; }
template <int N> SBZ_HD Tay<N> operator/(const Tay<N>& a, double b) { return a * (1.0 / b); }
template <int N> SBZ_HD Tay<N> operator*(const Tay<N>& a, const Tay<N>& b) {
  Tay<N> r;
#pragma unroll
  for (int k = 0; k <= N; ++k) {
    double s = 0;
#pragma unroll
    for (int j = 0; j <= k; ++j) s += a.c[j] * b.c[k - j];
    r.c[k] = s;
  }
  return r;
}
template <int N> SBZ_HD Tay<N> operator/(const Tay<N>& a, const Tay<N>& b) {
  Tay<N> r;
  const double ib = 1.0 / b.c[0];
#pragma unroll
  for (int k = 0; k <= N; ++k) {
    double s = a.c[k];
#pragma unroll
    for (int j = 1; j <= k; ++j) s -= b.c[j] * r.c[k - j];
    r.c[k] = s * ib;
  }
  return r;
}
template <int N> SBZ_HD Tay<N> operator/(double a, const Tay<N>& b) { return Tay<N>(a) / b; }
template <int N> SBZ_HD Tay<N>& operator+=(Tay<N>& a, const Tay<N>& b) { a = a + b; return a; }
template <int N> SBZ_HD Tay<N>& operator+=(Tay<N>& a, double b) { a.c[0] += b; return a; }

template <int N> SBZ_HD Tay<N> exp(const Tay<N>& u) {
  Tay<N> w; w.c[0] = ::exp(u.c[0]);
#pragma unroll
  for (int k = 1; k <= N; ++k) {
    double s = 0;
#pragma unroll
    for (int j = 1; j <= k; ++j) s += j * u.c[j] * w.c[k - j];
    w.c[k] = s / k;
  }
  return w;
}
template <int N> SBZ_HD Tay<N> log(const Tay<N>& u) {
  Tay<N> w; w.c[0] = ::log(u.c[0]);
#pragma unroll
  for (int k = 1; k <= N; ++k) {
    double s = 0;
#pragma unroll
    for (int j = 1; j < k; ++j) s += j * w.c[j] * u.c[k - j];
    w.c[k] = (u.c[k] - s / k) / u.c[0];
  }
  return w;
}
template <int N> SBZ_HD Tay<N> pow(const Tay<N>& u, double p) {
  Tay<N> w; w.c[0] = ::pow(u.c[0], p);
#pragma unroll
  for (int k = 1; k <= N; ++k) {
    double s = 0;
#pragma unroll
    for (int j = 0; j < k; ++j) s += (p * (k - j) - j) * u.c[k - j] * w.c[j];
    w.c[k] = s / (k * u.c[0]);
  }
  return w;
}
template <int N> SBZ_HD Tay<N> sqrt(const Tay<N>& u) { return pow(u, 0.5); }
template <int N> SBZ_HD Tay<N> tanh(const Tay<N>& u) {
  Tay<N> t, s; t.c[0] = ::tanh(u.c[0]); s.c[0] = 1.0 - t.c[0] * t.c[0];
#pragma unroll
  for (int k = 1; k <= N; ++k) {
    double a = 0, b = 0;
#pragma unroll
    for (int j = 1; j <= k; ++j) a += j * u.c[j] * s.c[k - j];
    t.c[k] = a / k;
#pragma unroll
    for (int j = 0; j <= k; ++j) b += t.c[j] * t.c[k - j];
    s.c[k] = -b;
  }
  return t;
}

SBZ_HD double exp(double x) { return ::exp(x); }
SBZ_HD double log(double x) { return ::log(x); }
SBZ_HD double pow(double x, double p) { return ::pow(x, p); }
SBZ_HD double sqrt(double x) { return ::sqrt(x); }
SBZ_HD double tanh(double x) { return ::tanh(x); }

template <class T> SBZ_HD double val(const T& x) { return x.c[0]; }
SBZ_HD double val(double x) { return x; }

}  // namespace sbz
