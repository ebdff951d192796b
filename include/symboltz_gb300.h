/* symboltz_gb300: C-ABI of the GB300 perturbation + line-of-sight engine.
 *
 * Drop-in for the hot path of hersle/SymBoltz.jl.  Each entry point names the reference
 * function (file:line inside the SymBoltz.jl repository) whose behaviour it replaces; a Julia
 * module binds them with ccall, the Python package symboltz with ctypes.
 *
 * Conventions: plain pointers and sizes; host pointers unless the name ends in _device;
 * integer status returns (0 = ok, < 0 = argument/CUDA errors, see SBZ_ERR_*); per-mode solver
 * failures never abort a call: they are reported per mode (SBZ_MAXITERS, SBZ_DTMIN,
 * SBZ_NONFINITE) exactly where the reference warns and returns a non-success retcode
 * (src/solve.jl:557-564).  One CUDA stream per problem handle; a handle is not re-entrant.
 * Units follow the reference: τ in 1/H0, k in H0/c (src/SymBoltz.jl:23-28).
 */
#ifndef SYMBOLTZ_GB300_H
#define SYMBOLTZ_GB300_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define SBZ_OK 0
#define SBZ_MAXITERS 1     /* more steps than opts.maxiters */
#define SBZ_DTMIN 2        /* step size underflow */
#define SBZ_NONFINITE 3    /* NaN/Inf in the solution or its error estimate */
#define SBZ_ERR_ARG (-1)
#define SBZ_ERR_CUDA (-2)
#define SBZ_ERR_NOMEM (-3)
#define SBZ_ERR_STATE (-4)

/* ---- stage linear solves ---- */
#define SBZ_FP64 0   /* structured LU of (1/(hγ) - J) in FP64 */
#define SBZ_MIXED 1  /* structured LU in FP32 + FP64 iterative refinement (FP64 residuals) */

/* ---- perturbation outputs ---- */
#define SBZ_OUT_SOURCES 0  /* k*S_T, k^2*S_E, S_psi at the saved times   (src/models/cosmologies.jl:99-105) */
#define SBZ_OUT_DELTA_M 1  /* total matter Δ_m(τ0)                         (src/observables/fourier.jl:39-52) */
#define SBZ_OUT_STATE 2    /* full perturbation state at the saved times   (solvept output_func = identity) */
#define SBZ_OUT_SOURCES4 3 /* k*S_T split into k*(SW + ISW), k*Doppler, k*polarisation, and k^2*S_E
                              (the four ST/SE terms of src/models/cosmologies.jl:99-104) */
#define SBZ_OUT_FACTORS 4  /* the perturbation factors of the sources: δγ/4 + Ψ + Π/16, Ψ' + Φ', θb, θb',
                              Π, Π', Π'' (S_T = v·f0 + e^{-κ} f1 + (v̇ f2 + v f3)/k² + 3(v̈ f4 + 2v̇ f5 + v f6)/(16k²),
                              S_E = 3 v f4 / (16 (kχ)²)) */

/* Cosmological parameters of one cosmology: parameters_Planck18 keys (src/parameters.jl:1-21). */
typedef struct sbz_params {
  double h, Omega_c, Omega_b, T0, Neff, YHe, ln_As1e10, ns;
  double m_nu_eV;  /* mass of each massive neutrino (eV) */
  double N_nu;     /* number of degenerate massive neutrinos */
} sbz_params;

/* Model options: ΛCDM(lmax, Hswitch, Heswitch, reionization) (src/models/cosmologies.jl:27-48). */
typedef struct sbz_model {
  int lmax_gamma;  /* photon temperature + polarisation hierarchy (>= 3) */
  int lmax_nu;     /* massless neutrinos (>= 3) */
  int lmax_h;      /* massive neutrinos (>= 3) */
  int nx_h;        /* massive-neutrino momentum bins (0 = no massive species, max 8) */
  int Hswitch, Heswitch, reionization;
} sbz_model;

/* Solver options: CosmologyProblem(ivspan) + solve(bgopts, ptopts) (src/solve.jl:129-134,380-386). */
typedef struct sbz_opts {
  double bg_rtol, bg_atol;  /* default 1e-7 */
  double pt_rtol, pt_atol;  /* default 1e-5 */
  double tau_ini, tau_max;  /* background span, default (1e-6, 100) */
  int64_t maxiters;         /* default 100000 */
  int precision;            /* SBZ_FP64 or SBZ_MIXED */
  int refine_iters;         /* SBZ_MIXED: at most this many FP64 refinement sweeps per stage solve, stopping
                               once a correction is < 1e-3 of the error tolerance; default 3 */
  int table_points;         /* background coefficient table nodes, default 8192 */
  int warps_per_block;      /* warps per thread block (≤ 4); 0 = 4 */
  int warps_per_mode;       /* warps integrating one mode: 1, 2, 4 or 8; 0 = chosen from the number of modes */
  int blocks_per_sm;        /* resident thread blocks per SM for the perturbation kernel; 0 = chosen */
  int los_precision;        /* line of sight: SBZ_FP64 or SBZ_MIXED (FP32 interpolation); -1 = as precision */
  double refine_skip;       /* SBZ_MIXED: the later stages (2-8) of a step are refined only when stage 1's
                               first correction is at or above this (error-weight units); stage 1 is always
                               refined.  0 = refine every stage; < 0 (default) = 1e-5 for four-warp groups
                               (sources at the fully refined accuracy) and 0 for narrower ones.  Larger
                               values trade pointwise source accuracy for speed: 1e-2 keeps the 1000-mode
                               massive-ν C_l within 7.4e-6 of the all-FP64 solver at rtol 1e-6, atol 3e-8
                               (2.01 s against 2.90 s at 1e-4), while skipping the later stages' refinement
                               outright leaves pointwise sources of the ΛCDM(lmax = 5) model 1e-2 off */
} sbz_opts;

typedef struct sbz_problem sbz_problem;
typedef struct sbz_bessel sbz_bessel;

void sbz_default_opts(sbz_opts* o);
const char* sbz_last_error(void);

/* Momentum bins x_i and weights W_i for ∫dx x² f0(x) g(x) (src/models/neutrinos.jl:55-60). */
int sbz_momentum_quadrature(int N, double* x, double* W);

/* CosmologyProblem(M, pars) for n_cosmo parameter sets sharing one model (src/solve.jl:129-236;
 * several sets replace the reference's parameter_updater loop, src/solve.jl:272-307). */
int sbz_problem_create(const sbz_model* m, const sbz_params* p, int n_cosmo, const sbz_opts* o, sbz_problem** out);
void sbz_problem_destroy(sbz_problem* pb);
int sbz_problem_nstate(const sbz_problem* pb);
/* Replace the parameter sets of an existing problem (batched parameter upload; the problem-level
 * form of parameter_updater, src/solve.jl:271-306).  The model, options, stream and device buffers
 * are kept (buffers grow when n_cosmo does); the background must be solved again before the next
 * perturbation call.  Waits for the problem's stream first. */
int sbz_problem_set_params(sbz_problem* pb, const sbz_params* p, int n_cosmo);

/* solvebg (src/solve.jl:427-435) with the a = 1 callback (src/solve.jl:158-203): τ0, κ0, τrec and
 * status per cosmology (arrays of n_cosmo, any may be NULL).  Also builds and uploads the
 * background coefficient tables read by the perturbation kernels. */
int sbz_solve_bg(sbz_problem* pb, double* tau0, double* kappa0, double* taurec, int* status);
/* Background solution knots of one cosmology (bgsol.t and unknowns); returns the count. */
int sbz_bg_knots(const sbz_problem* pb, int cosmo, int cap, double* tau, double* y5);
/* Derived background quantities (a, ℋ, κ̇, κ, v, v̇, c_s², Xe, Tb) at n times. */
int sbz_bg_eval(const sbz_problem* pb, int cosmo, int n, const double* tau, double* out9);

/* Background coefficients as the perturbation kernels read them (Hermite interpolation of the
 * per-cosmology table): a, ℋ, κ̇, c_s², e^{-κ}, κ̈, κ⃛ at n times (thermodynamics observables of
 * src/models/baryons.jl:155-183). */
int sbz_bg_coefficients(const sbz_problem* pb, int cosmo, int n, const double* tau, double* out7);

/* solvept (src/solve.jl:543-569) over nk modes: mode i belongs to cosmology cosmo[i] (NULL = all 0),
 * has wavenumber ks[i] and initial time tau_ini[i] (clamped to the background span, src/solve.jl:527).
 * Saved times: taus[c*ntau + j] for cosmology c (saveat).  out layout:
 *   SBZ_OUT_SOURCES: out[(i*ntau + j)*3 + s]; SBZ_OUT_DELTA_M: out[i]; SBZ_OUT_STATE: out[(i*ntau + j)*n + m];
 *   SBZ_OUT_SOURCES4: out[(i*ntau + j)*4 + s]; SBZ_OUT_FACTORS: out[(i*ntau + j)*7 + s].
 * status[i] per mode (may be NULL); steps[2i], steps[2i+1] = accepted, rejected (may be NULL). */
int sbz_solve_pt(sbz_problem* pb, int nk, const int* cosmo, const double* ks, const double* tau_ini,
                 int ntau, const double* taus, int output, double* out, int* status, int64_t* steps);
/* Same with device pointers, enqueued on the problem's stream (no host synchronisation). */
int sbz_solve_pt_device(sbz_problem* pb, int nk, const int* cosmo, const double* ks, const double* tau_ini,
                        int ntau, const double* taus, int output, double* out, int* status, int64_t* steps);

/* The perturbation right-hand side f = J(τ) y and ∂f/∂τ as the GPU integrator evaluates them, for
 * nk (cosmology, k, τ, y) points: the counterpart of the generated ODE function prob.pt.f and its
 * time derivative (src/solve.jl:227).  y, f, dfdtau: [i*n + m] in the library's state ordering
 * (see sbz_layout.hpp: Φ, δc, θc, δb, θb, F0-2, G0-2, F3.., G3.., N0.., ψ_{j,l}). */
int sbz_pt_rhs(sbz_problem* pb, int nk, const int* cosmo, const double* ks, const double* taus, const double* y,
               double* f, double* dfdtau);

/* spectrum_matter(prob, ks) (src/observables/fourier.jl:79-101): P(k, τ0) = P0(k) Δ_m² with
 * τ_ini = min(kτini/k, τinimax); kτini = 1e-2, τinimax = 1e-4 by default. */
int sbz_spectrum_matter(sbz_problem* pb, int nk, const int* cosmo, const double* ks, double ktau_ini,
                        double tau_ini_max, double* Pk, int* status);
/* spectrum_primordial (src/observables/fourier.jl:14-30) of one cosmology. */
int sbz_spectrum_primordial(const sbz_problem* pb, int cosmo, int nk, const double* ks, double* P0);

/* SphericalBesselCache(ls; xmax, dx, hermite) (src/observables/angular.jl:18-26), built on the GPU. */
int sbz_bessel_create(int nl, const int* ls, double xmax, double dx, int hermite, sbz_bessel** out);
void sbz_bessel_destroy(sbz_bessel* jl);
/* Interpolated j_l(x) from the cache for cache index il at n points (angular.jl:29-48). */
int sbz_bessel_eval(const sbz_bessel* jl, int il, int n, const double* x, double* out);

/* los_integrate(Ss, ls, τs, ks, jl; l_limber) (src/observables/angular.jl:109-185).
 * S[(it*nk + ik)*nsrc + s] -> out[(ik*nl + il)*nsrc + s]; l_limber applies to every source. */
int sbz_los_integrate(const sbz_bessel* jl, int nsrc, const double* S, int ntau, const double* taus,
                      int nk, const double* ks, int l_limber, double* out);
int sbz_los_integrate_device(const sbz_bessel* jl, int nsrc, const double* S, int ntau, const double* taus,
                             int nk, const double* ks, int l_limber, double* out, void* stream);

/* k-interpolation of the sources (src/observables/fourier.jl:227-247,464-547) */
#define SBZ_KINTERP_SPLINE 0       /* natural cubic spline in y = f(k) (CubicSplineInterpolator) */
#define SBZ_KINTERP_BARYCENTRIC 1  /* barycentric formula with weights w in y = f(k) (ChebyshevInterpolator) */

/* spectrum_cmb(modes, prob, jl) (src/observables/angular.jl:260-341) as one device pipeline with host
 * inputs and outputs: solve the nc coarse modes of cosmology `cosmo` from the background start
 * with sources saved at taus (source_grid, fourier.jl:267-291), interpolate them to the fine grid
 * ks_fine (y-values yc/yf = f(k); weights wc for SBZ_KINTERP_BARYCENTRIC), zero the last time,
 * line-of-sight integrate over the cache's l (T and E without Limber, ψ with l_limber), scale
 * Θ_T and Θ_E, and integrate C_l for npair source pairs (0 = T, 1 = E, 2 = ψ):
 * out_cl[q*nl + il].  status[nc] receives the per-mode solver status (may be NULL). */
int sbz_spectrum_cmb(sbz_problem* pb, int cosmo, const sbz_bessel* jl, int nc, const double* ks_coarse, const double* yc,
                     const double* wc, int interp, int ntau, const double* taus, int nf, const double* ks_fine,
                     const double* yf, int npair, const int* pair_a, const int* pair_b, int l_limber, double* out_cl,
                     int* status);
/* sbz_spectrum_cmb with the coarse sources supplied by the caller instead of the perturbation
 * solve (no counterpart in the reference; used for surrogate sources): sources[(i*ntau + j)*3 + s]
 * = (k S_T, k² S_E, S_ψ) at ks_coarse[i], taus[j], the SBZ_OUT_SOURCES layout. */
int sbz_spectrum_cmb_sources(sbz_problem* pb, int cosmo, const sbz_bessel* jl, int nc, const double* ks_coarse, const double* yc,
                             const double* wc, int interp, int ntau, const double* taus, const double* sources, int nf,
                             const double* ks_fine, const double* yf, int npair, const int* pair_a, const int* pair_b, int l_limber,
                             double* out_cl);
/* Launch everything of this problem on an external CUDA stream (NULL: back to an own stream). */
int sbz_problem_set_stream(sbz_problem* pb, void* stream);
/* CUDA-event durations (ms) of the last sbz_spectrum_cmb: H2D, perturbations, k-interpolation,
 * line of sight, C_l, D2H, total, (reserved). */
int sbz_problem_timings(const sbz_problem* pb, double* ms8);

/* No counterpart in the reference (its solvept threads over k on the CPU).  Autotuner for the
 * perturbation kernel's launch shape: times the candidates (warps per mode, blocks per SM) =
 * (1,0) (2,0) (2,2) (4,1) (4,2) (4,3) (8,1) on a k-stratified sample of the given modes (an eighth of
 * them above 2048 modes, all of them otherwise), stores the fastest in the problem's options and
 * returns it in best[2]; ms[SBZ_TUNE_CANDIDATES] receives the candidates' kernel times (may be
 * NULL).  Arguments as sbz_solve_pt. */
#define SBZ_TUNE_CANDIDATES 7
int sbz_autotune_pt(sbz_problem* pb, int nk, const int* cosmo, const double* ks, const double* tau_ini, int ntau,
                    const double* taus, int output, int* best, double* ms);

/* No counterpart in the reference: the source surrogate's dense-layer GEMM (BF16 tcgen05 tensor
 * cores, FP32 accumulation), exposed for testing.  D = A·Bᵀ with A [M][K] and B [N][K] bf16
 * row-major device matrices (16-byte aligned; M % 128 == 0, N % 64 == 0, K % 64 == 0), then
 *   epi SBZ_MLP_F32:  out (float, row stride ldo) = D, or += D when accumulate;
 *   epi SBZ_MLP_ACT:  z = D + bias; out (bf16) = act(z); z_out (bf16, may be NULL) = z;
 *   epi SBZ_MLP_DACT: out (bf16) = D · act'(z_in);
 * act SBZ_MLP_NONE or SBZ_MLP_SILU; only columns < n_valid (0: N) are written.  Queued on
 * `stream`; the call waits for it and reports a pipeline timeout as SBZ_ERR_CUDA. */
#define SBZ_MLP_F32 0
#define SBZ_MLP_ACT 1
#define SBZ_MLP_DACT 2
#define SBZ_MLP_NONE 0
#define SBZ_MLP_SILU 1
int sbz_mlp_gemm(int M, int N, int K, const void* A, const void* B, int epi, int act, const float* bias, void* out, int ldo,
                 int n_valid, int accumulate, void* z_out, const void* z_in, void* stream);

/* Source surrogate (sbz_surrogate_*; a learned part with no counterpart in the reference):
 * an MLP nin → nhidden × width (SiLU) → nout trained and evaluated with the BF16 tensor-core GEMM
 * above (FP32 accumulation, FP32 master weights, Adam, MSE loss on the caller's normalised targets).
 * nin, nout ≤ 64, width % 128 == 0, batch % 128 == 0.  Inputs/targets are host float arrays
 * X[n][nin], Y[n][nout].  Parameters in flat order: per layer W[nout][nin] then b[nout]. */
typedef struct sbz_surrogate sbz_surrogate;
int sbz_surrogate_create(int nin, int width, int nhidden, int nout, int batch, unsigned long long seed, sbz_surrogate** out);
void sbz_surrogate_destroy(sbz_surrogate* s);
long long sbz_surrogate_nparams(const sbz_surrogate* s);
int sbz_surrogate_get_params(const sbz_surrogate* s, float* params);
int sbz_surrogate_set_params(sbz_surrogate* s, const float* params);
/* Copy a training set to the device (replaces the previous one). */
int sbz_surrogate_set_data(sbz_surrogate* s, long long n, const float* X, const float* Y);
/* nsteps Adam steps (β = 0.9, 0.999) on batches drawn uniformly with replacement; *loss = mean
 * squared error of the last batch. */
int sbz_surrogate_train(sbz_surrogate* s, int nsteps, double lr, double* loss);
/* Forward pass and gradients (flat parameter order) of the mean squared error on exactly these
 * n rows (n % 128 == 0, n ≤ batch); the weights are not changed. */
int sbz_surrogate_gradients(sbz_surrogate* s, int n, const float* X, const float* Y, double* loss, float* grads);
int sbz_surrogate_infer(sbz_surrogate* s, long long n, const float* X, float* Y);
/* Flat binary weight file: "SBZMLP01", int32 nin, width, nhidden, nout, FP32 parameters. */
int sbz_surrogate_save(const sbz_surrogate* s, const char* path);
int sbz_surrogate_load(const char* path, int batch, sbz_surrogate** out);
/* Flat binary training-set file: "SBZTRN01", int32 nin, int32 nout, int64 nrows, then nrows rows of
 * nin + nout float32 (inputs, then targets).  The data side of the surrogate's I/O; the reference
 * has no surrogate, its batched parameter path (parameter_updater, src/solve.jl:271-306) is what
 * produces the data.  _append creates the file or adds rows to it (the shapes must match);
 * _read copies rows [first, first + n). */
int sbz_trainset_append(const char* path, int nin, int nout, long long n, const float* X, const float* Y);
int sbz_trainset_info(const char* path, int* nin, int* nout, long long* nrows);
int sbz_trainset_read(const char* path, long long first, long long n, float* X, float* Y);

/* spectrum_cmb(ΘlAs, ΘlBs, P0s, ls, ks) (src/observables/angular.jl:198-223): natural cubic
 * spline through (0,0) and (k, 2/π k² P0 Θ_A Θ_B), integrated exactly.  Th[ik*nl + il]. */
int sbz_cl_integrate(int nk, const double* ks, const double* P0, int nl, const double* ThA,
                     const double* ThB, double* Cl);

/* No counterpart in the reference.  sbz_cl_integrate on device buffers that allocates no device
 * memory, for callers whose memory belongs to their own pool (CUDA.jl, PyTorch's caching
 * allocator, a fixed serving budget) and who must not see cudaMalloc/cudaFree, which sit outside
 * that pool and synchronise the device.  d_ks, d_P0, d_ThA, d_ThB (Th[ik*nl + il]) and d_Cl[nl]
 * are device pointers; the work is queued on `stream` (NULL: the default stream) and the call
 * returns without waiting.  Scratch is a fixed SBZ_NOALLOC_SCRATCH_DOUBLES-double device array:
 * sizes with 2*ceil32(nk+1) + (nk+1)*nl above it return SBZ_ERR_ARG.  All calls share that array
 * (it keeps the last call's contents), so calls that overlap on the GPU race.  Every call looks up
 * the array's address in the current context; the first call on a device also loads the module
 * there, so make it before any stream capture.  Knots that are not
 * positive and increasing give NaN C_l (the host does not read device inputs). */
#define SBZ_NOALLOC_SCRATCH_DOUBLES 2097152
int sbz_cl_integrate_noalloc(int nk, const double* d_ks, const double* d_P0, int nl, const double* d_ThA,
                             const double* d_ThB, double* d_Cl, void* stream);

#ifdef __cplusplus
}
#endif
#endif
