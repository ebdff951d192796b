// CPU oracle, line-of-sight part.  TEST INFRASTRUCTURE ONLY (see oracle.h).
//
//   spherical Bessel j_l(x)          reference: Bessels.jl sphericalbesselj (not vendored), used at
//                                    src/observables/angular.jl:59; restated here by recurrences
//   SphericalBesselCache + eval      src/observables/angular.jl:9-48
//   los_integrate (incl. Limber)     src/observables/angular.jl:109-185
//   spectrum_cmb k-integral          src/observables/angular.jl:198-223 (natural cubic spline integral)
//   natural cubic spline             DataInterpolations.CubicSpline (not vendored), used at
//                                    src/observables/angular.jl:212-213,356
#include "oracle.h"
#include <vector>
#include <cmath>
#include <cstring>
#include <algorithm>

namespace {

// j_l(x) for l = 0..L at one x.  Upward recurrence where it is stable (l < x), Miller's
// downward recurrence (normalised by j_0 or j_1) otherwise, with rescaling against overflow.
void sph_bessel_all(int L, double x, double* out) {
  if (x == 0.0) { out[0] = 1.0; for (int l = 1; l <= L; ++l) out[l] = 0.0; return; }
  const double s = std::sin(x), c = std::cos(x);
  const double j0 = s / x, j1 = (s / x - c) / x;
  if (L == 0) { out[0] = j0; return; }
  if (x > L) {
    out[0] = j0; out[1] = j1;
    for (int l = 1; l < L; ++l) out[l + 1] = (2 * l + 1) / x * out[l] - out[l - 1];
    return;
  }
  const int Ls = L + 30 + (int)std::sqrt(40.0 * (L + 1));
  std::vector<double> t(Ls + 2, 0.0);
  t[Ls + 1] = 0.0; t[Ls] = 1e-300;
  for (int l = Ls; l >= 1; --l) {
    t[l - 1] = (2 * l + 1) / x * t[l] - t[l + 1];
    if (std::fabs(t[l - 1]) > 1e200) {
      for (int m = l - 1; m <= Ls + 1; ++m) t[m] *= 1e-200;
    }
  }
  const double norm = (std::fabs(j0) >= std::fabs(j1)) ? j0 / t[0] : j1 / t[1];
  for (int l = 0; l <= L; ++l) out[l] = t[l] * norm;
}

struct Spline {  // natural cubic spline second derivatives
  static void second(int n, const double* x, const double* y, double* z) {
    std::vector<double> a(n), b(n), c(n), d(n);
    z[0] = z[n - 1] = 0;
    if (n < 3) { for (int i = 0; i < n; ++i) z[i] = 0; return; }
    // equations for i = 1..n-2:  h_{i-1} z_{i-1} + 2(h_{i-1}+h_i) z_i + h_i z_{i+1} = 6(dy_i/h_i - dy_{i-1}/h_{i-1})
    int m = n - 2;
    std::vector<double> sub(m), dia(m), sup(m), rhs(m);
    for (int i = 1; i <= m; ++i) {
      double h0 = x[i] - x[i - 1], h1 = x[i + 1] - x[i];
      sub[i - 1] = h0; dia[i - 1] = 2 * (h0 + h1); sup[i - 1] = h1;
      rhs[i - 1] = 6 * ((y[i + 1] - y[i]) / h1 - (y[i] - y[i - 1]) / h0);
    }
    for (int i = 1; i < m; ++i) { double w = sub[i] / dia[i - 1]; dia[i] -= w * sup[i - 1]; rhs[i] -= w * rhs[i - 1]; }
    z[m] = rhs[m - 1] / dia[m - 1];
    for (int i = m - 2; i >= 0; --i) z[i + 1] = (rhs[i] - sup[i] * z[i + 2]) / dia[i];
  }
};

}  // namespace

struct orc_jl {
  std::vector<int> l;
  std::vector<double> y, dy;  // [ix * nl + il]
  double dx, invdx, xmax; int nx; int hermite;
};

extern "C" void orc_sph_bessel(int nl, const int* ls, int nx, const double* x, double* out) {
  int L = 0; for (int i = 0; i < nl; ++i) L = std::max(L, ls[i]);
#pragma omp parallel
  {
    std::vector<double> buf(L + 2);
#pragma omp for
    for (int i = 0; i < nx; ++i) {
      sph_bessel_all(L, x[i], buf.data());
      for (int j = 0; j < nl; ++j) out[(size_t)i * nl + j] = buf[ls[j]];
    }
  }
}

extern "C" orc_jl* orc_jl_create(int nl, const int* ls, double xmax, double dx, int hermite) {
  orc_jl* c = new orc_jl();
  c->l.assign(ls, ls + nl);
  const int N = (int)std::trunc(xmax / dx);  // range(0, xmax, length = trunc(xmax/dx))
  const double step = xmax / (N - 1);
  c->dx = dx; c->invdx = 1.0 / step; c->xmax = xmax; c->nx = N + 1; c->hermite = hermite;
  c->y.assign((size_t)c->nx * nl, 0.0);
  if (hermite) c->dy.assign((size_t)c->nx * nl, 0.0);
  int L = 0; for (int v : c->l) L = std::max(L, v);
#pragma omp parallel
  {
    std::vector<double> buf(L + 3);
#pragma omp for schedule(dynamic, 64)
    for (int ix = 0; ix < N; ++ix) {
      const double x = (ix == N - 1) ? xmax : ix * step;
      sph_bessel_all(L + 1, x, buf.data());
      for (int il = 0; il < nl; ++il) {
        const int l = c->l[il];
        c->y[(size_t)ix * nl + il] = buf[l];
        if (hermite) c->dy[(size_t)ix * nl + il] = (l == 0) ? -buf[1] : (l * buf[l - 1] - (l + 1) * buf[l + 1]) / (2.0 * l + 1);
      }
    }
  }
  // duplicated last point (avoids a bounds check in the interpolation)
  for (int il = 0; il < nl; ++il) {
    c->y[(size_t)N * nl + il] = c->y[(size_t)(N - 1) * nl + il];
    if (hermite) c->dy[(size_t)N * nl + il] = c->dy[(size_t)(N - 1) * nl + il];
  }
  return c;
}
extern "C" void orc_jl_free(orc_jl* c) { delete c; }
extern "C" int orc_jl_nx(const orc_jl* c) { return c->nx; }
extern "C" double orc_jl_xmax(const orc_jl* c) { return c->xmax; }

static inline double jl_eval(const orc_jl* c, int il, double x) {
  const int nl = (int)c->l.size();
  double w = x * c->invdx;
  int i = (int)w;
  w -= i;
  const double ym = c->y[(size_t)i * nl + il], yp = c->y[(size_t)(i + 1) * nl + il];
  if (!c->hermite) return ym + w * (yp - ym);
  const double dym = c->dy[(size_t)i * nl + il], dyp = c->dy[(size_t)(i + 1) * nl + il];
  const double wm1 = w - 1.0;
  // the reference scales the slopes by the requested dx (not the realised grid step)
  return (1 + 2 * w) * wm1 * wm1 * ym + w * w * (3 - 2 * w) * yp + w * wm1 * (wm1 * dym + w * dyp) * c->dx;
}

extern "C" void orc_jl_eval(const orc_jl* c, int il, int n, const double* x, double* out) {
  for (int i = 0; i < n; ++i) out[i] = jl_eval(c, il, x[i]);
}

extern "C" int orc_los_integrate(const orc_jl* c, int nsrc, const double* S, int ntau, const double* taus,
                                 int nk, const double* ks, int l_limber, double* out) {
  const int nl = (int)c->l.size();
  const double tau0 = taus[ntau - 1];
  std::vector<double> chi(ntau), w(ntau);
  for (int i = 0; i < ntau; ++i) chi[i] = tau0 - taus[i];
  w[0] = 0.5 * (taus[1] - taus[0]);
  for (int i = 1; i < ntau - 1; ++i) w[i] = 0.5 * (taus[i + 1] - taus[i - 1]);
  w[ntau - 1] = 0.5 * (taus[ntau - 1] - taus[ntau - 2]);
  int il_limber = nl;
  for (int il = 0; il < nl; ++il) if (c->l[il] >= l_limber) { il_limber = il; break; }
#pragma omp parallel
  {
    std::vector<double> tmp((size_t)nl * nsrc);
#pragma omp for schedule(dynamic, 4)
    for (int ik = 0; ik < nk; ++ik) {
      const double k = ks[ik];
      std::fill(tmp.begin(), tmp.end(), 0.0);
      for (int it = 0; it < ntau; ++it) {
        const double kchi = k * chi[it];
        double Sw[8];
        for (int s = 0; s < nsrc; ++s) Sw[s] = w[it] * S[((size_t)it * nk + ik) * nsrc + s];
        for (int il = 0; il < il_limber; ++il) {
          const double j = jl_eval(c, il, kchi);
          for (int s = 0; s < nsrc; ++s) tmp[(size_t)il * nsrc + s] += Sw[s] * j;
        }
      }
      // Limber approximation for l >= l_limber (src/observables/angular.jl:154-178)
      for (int il = il_limber; il < nl; ++il) {
        const double l = c->l[il];
        const double x = (l + 0.5) / k;
        if (!(x <= chi[0])) continue;
        // first index with taus[i] >= tau0 - x
        int im = (int)(std::lower_bound(taus, taus + ntau, tau0 - x) - taus);
        if (im == 0) continue;  // the reference leaves the integral at zero here
        const int ip = im - 1;
        const double chim = chi[im], chip = chi[ip], dchi = chip - chim;
        for (int s = 0; s < nsrc; ++s) {
          auto Sv = [&](int i) { return S[((size_t)i * nk + ik) * nsrc + s]; };
          const double Sm = Sv(im), Sp = Sv(ip);
          const double dSm = (im <= ntau - 2) ? (Sv(im + 1) - Sp) / (chi[im + 1] - chip) : (Sp - Sm) / dchi;
          const double dSp = (ip >= 1) ? (Sm - Sv(im - 2 >= 0 ? im - 2 : 0)) / (chim - chi[im - 2 >= 0 ? im - 2 : 0]) : (Sp - Sm) / dchi;
          const double t = (x - chim) / dchi, t2 = t * t, t3 = t2 * t;
          const double Sx = (2 * t3 - 3 * t2 + 1) * Sm + (t3 - 2 * t2 + t) * dchi * dSm + (-2 * t3 + 3 * t2) * Sp + (t3 - t2) * dchi * dSp;
          tmp[(size_t)il * nsrc + s] = std::sqrt(M_PI / (2 * l + 1)) * Sx / k;
        }
      }
      std::memcpy(out + (size_t)ik * nl * nsrc, tmp.data(), sizeof(double) * nl * nsrc);
    }
  }
  return 0;
}

extern "C" void orc_cl_integrate(int nk, const double* ks, const double* P0, int nl, const double* ThA,
                                 const double* ThB, double* Cl) {
#pragma omp parallel
  {
    std::vector<double> x(nk + 1), y(nk + 1), z(nk + 1);
#pragma omp for
    for (int il = 0; il < nl; ++il) {
      x[0] = 0; y[0] = 0;
      for (int ik = 0; ik < nk; ++ik) {
        x[ik + 1] = ks[ik];
        y[ik + 1] = 2 / M_PI * ks[ik] * ks[ik] * P0[ik] * ThA[(size_t)ik * nl + il] * ThB[(size_t)ik * nl + il];
      }
      Spline::second(nk + 1, x.data(), y.data(), z.data());
      double s = 0;
      for (int i = 0; i < nk; ++i) {
        const double h = x[i + 1] - x[i];
        s += h * (y[i] + y[i + 1]) / 2 - h * h * h * (z[i] + z[i + 1]) / 24;
      }
      Cl[il] = s;
    }
  }
}

extern "C" void orc_cubic_spline(int n, const double* x, const double* y, int nq, const double* xq, double* out) {
  std::vector<double> z(n);
  Spline::second(n, x, y, z.data());
  for (int q = 0; q < nq; ++q) {
    const double t = xq[q];
    int i = (int)(std::upper_bound(x, x + n, t) - x) - 1;
    i = std::max(0, std::min(i, n - 2));
    const double h = x[i + 1] - x[i];
    const double A = x[i + 1] - t, B = t - x[i];
    out[q] = z[i] * A * A * A / (6 * h) + z[i + 1] * B * B * B / (6 * h) + (y[i + 1] / h - z[i + 1] * h / 6) * B + (y[i] / h - z[i] * h / 6) * A;
  }
}

// m natural cubic splines through (x, Y[:, c]) evaluated at xq, columns in parallel:
// Y[i * m + c] -> out[q * m + c] (the k-interpolation of the sources, one spline per (τ, source)).
extern "C" void orc_cubic_spline_columns(int n, const double* x, int m, const double* Y, int nq, const double* xq, double* out) {
  std::vector<int> iv(nq);
  for (int q = 0; q < nq; ++q) {
    int i = (int)(std::upper_bound(x, x + n, xq[q]) - x) - 1;
    iv[q] = std::max(0, std::min(i, n - 2));
  }
#pragma omp parallel
  {
    std::vector<double> y(n), z(n);
#pragma omp for schedule(static)
    for (int c = 0; c < m; ++c) {
      for (int i = 0; i < n; ++i) y[i] = Y[(size_t)i * m + c];
      Spline::second(n, x, y.data(), z.data());
      for (int q = 0; q < nq; ++q) {
        const int i = iv[q];
        const double t = xq[q], h = x[i + 1] - x[i], A = x[i + 1] - t, B = t - x[i];
        out[(size_t)q * m + c] = z[i] * A * A * A / (6 * h) + z[i + 1] * B * B * B / (6 * h) + (y[i + 1] / h - z[i + 1] * h / 6) * B +
                                 (y[i] / h - z[i] * h / 6) * A;
      }
    }
  }
}
