/* CPU oracle for the SymBoltz perturbation + line-of-sight path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is an independent FP64 restatement of the reference's
 * equations (hersle/SymBoltz.jl, src/models/ (all files), src/solve.jl, src/utils.jl,
 * src/observables/ (fourier.jl, angular.jl)).  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * may load it, and only as the checker.  The product library never links or calls it.
 *
 * Parity is pinned by the reference's own fixtures (test/class_Pk.dat, test/class_Cl.dat,
 * CLASS outputs for the reference's ΛCDM(lmax=5) + Planck18 case) and by the published momentum
 * quadrature table (paper/aa57450-25.tex:1370-1395); see tests/test_oracle_golden.py.
 */
#ifndef SBZ_ORACLE_H
#define SBZ_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_params {
  double h, Omega_c, Omega_b, T0, Neff, YHe, ln_As1e10, ns;
  double m_nu_eV;   /* mass of one massive neutrino (eV) */
  double N_nu;      /* degeneracy (number of equal-mass species) */
} orc_params;

typedef struct orc_model {
  int lmax_g, lmax_nu, lmax_h;  /* hierarchy truncations (photons T+P, massless nu, massive nu) */
  int nx;                       /* massive-nu momentum bins; 0 = no massive neutrinos */
  int Hswitch, Heswitch, reionization;
} orc_model;

typedef struct orc_opts {
  double bg_rtol, bg_atol, pt_rtol, pt_atol;
  double tau_ini, tau_max;      /* background integration span (src/solve.jl:131 ivspan) */
  long maxiters;
  int nthreads;
  int alg_bg, alg_pt;           /* ORC_RODAS4 or ORC_RODAS5P for the background / perturbations */
  int pt_linsolve;              /* ORC_LINSOLVE_DENSE (the checker) or ORC_LINSOLVE_SPARSE (CPU baseline) */
} orc_opts;

enum { ORC_RODAS4 = 0, ORC_RODAS5P = 1 };
enum { ORC_LINSOLVE_DENSE = 0, ORC_LINSOLVE_SPARSE = 1 };

/* Background solution handle. */
typedef struct orc_bg orc_bg;

int orc_momentum_quadrature(int N, double* x, double* W);
orc_bg* orc_bg_solve(const orc_params* p, const orc_model* m, const orc_opts* o, int* status);
void orc_bg_free(orc_bg* b);
/* info: tau0, kappa0, taurec, Omega_g0, Omega_nu0, Omega_h0, Omega_L0, nknots, fHe, As, kpivot, y0, Irho0 */
void orc_bg_info(const orc_bg* b, double* info);
int orc_bg_nknots(const orc_bg* b);
void orc_bg_knots(const orc_bg* b, double* tau, double* y /* nknots x 5 */);
/* Derived background quantities at times tau (from the Hermite spline of the 5 unknowns):
 * columns a, Hconf, kappa_dot, kappa, v, v_dot, cs2, Xe, Tb, XHe++ */
void orc_bg_eval(const orc_bg* b, int n, const double* tau, double* out /* n x 10 */);

/* Perturbation modes.
 * tau_ini[i] is the initial time for ks[i] (clamped to the background span).
 * mode 0: sources (k*S_T, k^2*S_E, S_psi) at ntau output times -> out[(ik*ntau + it)*3 + s]
 * mode 1: final-time total matter Delta_m(tau0) -> out[ik] (spectrum_matter without P0)
 * mode 2: full state at the ntau output times -> out[(ik*ntau + it)*n + i]
 * status[ik]: 0 ok, 1 maxiters, 2 dt underflow, 3 non-finite
 * stats[ik*2 + 0/1] = accepted / rejected steps. */
int orc_pt_nstate(const orc_model* m);
int orc_pt_solve(const orc_bg* b, int nk, const double* ks, const double* tau_ini, int ntau,
                 const double* taus, int mode, double* out, int* status, long* stats);
/* Right-hand side f = J(tau) y, dense J (n x n, row-major) and df/dtau of one mode (J may be NULL). */
int orc_pt_rhs(const orc_bg* b, double k, double tau, const double* y, double* f, double* J, double* ft);
/* Initial conditions of one mode at tau: state (n) plus Phi/Psi and f_nu */
int orc_pt_initial(const orc_bg* b, double k, double tau, double* y, double* extra);

/* Spherical Bessel j_l(x) for integer l >= 0 (own recurrence implementation). */
void orc_sph_bessel(int nl, const int* ls, int nx, const double* x, double* out /* nx x nl */);
/* Spherical Bessel cache (src/observables/angular.jl:18-26) and its interpolated evaluation. */
typedef struct orc_jl orc_jl;
orc_jl* orc_jl_create(int nl, const int* ls, double xmax, double dx, int hermite);
void orc_jl_free(orc_jl* c);
int orc_jl_nx(const orc_jl* c);
double orc_jl_xmax(const orc_jl* c);
void orc_jl_eval(const orc_jl* c, int il, int n, const double* x, double* out);
/* Line-of-sight integrals (src/observables/angular.jl:109-185).
 * S: nsrc sources, S[(it*nk + ik)*nsrc + s]; out I[(ik*nl + il)*nsrc + s] */
int orc_los_integrate(const orc_jl* c, int nsrc, const double* S, int ntau, const double* taus,
                      int nk, const double* ks, int l_limber, double* out);
/* C_l = int dk (2/pi) k^2 P0 ThA ThB with a natural cubic spline through (0,0)
 * (src/observables/angular.jl:198-223). ThA/ThB: [ik*nl + il] */
void orc_cl_integrate(int nk, const double* ks, const double* P0, int nl, const double* ThA,
                      const double* ThB, double* Cl);
/* Natural cubic spline through (x,y) evaluated at xq (DataInterpolations CubicSpline). */
void orc_cubic_spline(int n, const double* x, const double* y, int nq, const double* xq, double* out);
/* m such splines at once, columns of Y[i * m + c] -> out[q * m + c] (OpenMP over columns). */
void orc_cubic_spline_columns(int n, const double* x, int m, const double* Y, int nq, const double* xq, double* out);

#ifdef __cplusplus
}
#endif
#endif
