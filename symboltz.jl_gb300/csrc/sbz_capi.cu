// C-ABI entry points (include/symboltz_gb300.h).
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "../../include/symboltz_gb300.h"
#include "sbz_background.hpp"
#include "sbz_setup.hpp"
#include "sbz_pt.cuh"
#include "sbz_los.cuh"

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define SBZ_CUDA(call)                                                                          \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess) return fail(SBZ_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
  } while (0)

// Grow-only device buffer owned by a handle.
struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr; cap = 0;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e == cudaSuccess) cap = bytes;
    return e;
  }
  void release() { if (p) cudaFree(p); p = nullptr; cap = 0; }
  template <class T> T* as() const { return static_cast<T*>(p); }
};

// natural-spline Thomas factors for points X[0..n-1] (interior rows 1..n-2)
void spline_factors(const std::vector<double>& X, std::vector<double>& cprime, std::vector<double>& invden) {
  const int n = (int)X.size();
  cprime.assign(n, 0.0); invden.assign(n, 0.0);
  for (int i = 1; i <= n - 2; ++i) {
    const double h0 = X[i] - X[i - 1], h1 = X[i + 1] - X[i];
    invden[i] = 1.0 / (2 * (h0 + h1) - h0 * (i > 1 ? cprime[i - 1] : 0.0));
    cprime[i] = h1 * invden[i];
  }
}

template <class T>
cudaError_t up(DevBuf& b, const T* h, size_t n, cudaStream_t st) {
  cudaError_t e = b.ensure(sizeof(T) * std::max<size_t>(n, 1));
  if (e != cudaSuccess || n == 0) return e;
  return cudaMemcpyAsync(b.p, h, sizeof(T) * n, cudaMemcpyHostToDevice, st);
}

// Weights w with ∫ S = Σ_i w_i y_i for the natural cubic spline S through (X_i, y_i): the integral
// aᵀy - cᵀz of the spline (z = second derivatives, T z = R y) is (a - Rᵀ T⁻¹ c)ᵀ y, so one
// tridiagonal solve with the symmetric T gives the weights for every integrand on this grid.
void spline_integral_weights(const std::vector<double>& X, std::vector<double>& w) {
  const int n = (int)X.size();
  w.assign(n, 0.0);
  std::vector<double> h(n - 1);
  for (int i = 0; i + 1 < n; ++i) { h[i] = X[i + 1] - X[i]; w[i] += 0.5 * h[i]; w[i + 1] += 0.5 * h[i]; }
  const int m = n - 2;  // interior second derivatives z_1..z_{n-2}
  if (m < 1) return;
  std::vector<double> cp(m), v(m);
  for (int j = 0; j < m; ++j) {  // Thomas on T v = c, T_jj = 2(h_{i-1}+h_i), T_j,j+1 = h_i (i = j+1)
    const int i = j + 1;
    const double c = (h[i - 1] * h[i - 1] * h[i - 1] + h[i] * h[i] * h[i]) / 24.0;
    const double den = 2.0 * (h[i - 1] + h[i]) - (j > 0 ? h[i - 1] * cp[j - 1] : 0.0);
    cp[j] = h[i] / den;
    v[j] = (c - (j > 0 ? h[i - 1] * v[j - 1] : 0.0)) / den;
  }
  for (int j = m - 2; j >= 0; --j) v[j] -= cp[j] * v[j + 1];
  for (int j = 0; j < m; ++j) {  // w -= Rᵀ v,  R y = 6 ((y_{i+1}-y_i)/h_i - (y_i-y_{i-1})/h_{i-1})
    const int i = j + 1;
    w[i - 1] -= 6.0 / h[i - 1] * v[j];
    w[i] += 6.0 * (1.0 / h[i - 1] + 1.0 / h[i]) * v[j];
    w[i + 1] -= 6.0 / h[i] * v[j];
  }
}

int los_weights(const double* taus, int ntau, std::vector<double>& chi, std::vector<double>& w) {
  chi.resize(ntau); w.resize(ntau);
  const double t0 = taus[ntau - 1];
  for (int i = 0; i < ntau; ++i) chi[i] = t0 - taus[i];
  w[0] = 0.5 * (taus[1] - taus[0]);
  for (int i = 1; i < ntau - 1; ++i) w[i] = 0.5 * (taus[i + 1] - taus[i - 1]);
  w[ntau - 1] = 0.5 * (taus[ntau - 1] - taus[ntau - 2]);
  return SBZ_OK;
}

}  // namespace

namespace sbz {
// device build of the coefficient tables (sbz_table.cu)
int table_build_launch(int ntab, int ncos, const Cosmo* d_cosmo, const BgKnot* d_knots, const int* d_koff, const int* d_nknot,
                       const double* d_kappa0, const double* d_tabtau, const int* d_ok, double* d_tab, long long stride,
                       cudaStream_t stream);
}  // namespace sbz

struct sbz_problem {
  sbz_model model{};
  sbz_opts opts{};
  int ncosmo = 0;
  std::vector<sbz_params> params;
  std::vector<sbz::Background> bgs;
  std::vector<int> bg_status;
  sbz::ModelDesc M{};
  std::vector<sbz::CompDesc> comps;
  std::vector<sbz::CosmoDesc> cds;
  bool bg_done = false;
  bool tables_uploaded = false;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  DevBuf d_model, d_comps, d_cosmos, d_tables, d_counter;
  DevBuf d_k, d_ti, d_cosmo, d_order, d_taus, d_out, d_status, d_steps;
  DevBuf c_y, c_yf, c_iv, c_cp, c_id, c_z, c_Sf, c_Sp, c_ks, c_ls, c_Th, c_Thp, c_P0, c_cz, c_cl, c_pa, c_pb, c_src, c_M,
      c_chi, c_w, c_taus, c_kf;
  DevBuf t_cos, t_knots, t_koff, t_nknot, t_kap, t_tau, t_ok;  // inputs of the device table build
  int64_t table_stride = 0;
  bool own_stream = true;
  cudaEvent_t ev[12] = {};
  double timings[8] = {};
};

namespace {
enum { T_H2D = 0, T_PT, T_KINTERP, T_LOS, T_CL, T_D2H, T_TOTAL };
}

struct sbz_bessel {
  sbz::BesselDev J{};
  std::vector<int> ls;
  DevBuf d_y, d_dy, d_yf2, d_ls;
  DevBuf d_S, d_taus, d_chi, d_w, d_ks, d_out;
  cudaStream_t stream = nullptr;
};

extern "C" {

void sbz_default_opts(sbz_opts* o) {
  o->bg_rtol = 1e-7; o->bg_atol = 1e-7; o->pt_rtol = 1e-5; o->pt_atol = 1e-5;
  o->tau_ini = 1e-6; o->tau_max = 100.0; o->maxiters = 100000;
  o->precision = SBZ_MIXED; o->refine_iters = 3; o->table_points = 8192; o->warps_per_block = 0; o->warps_per_mode = 0; o->blocks_per_sm = 0;
  o->los_precision = -1; o->refine_skip = -1.0;
}

const char* sbz_last_error(void) { return g_err.c_str(); }

int sbz_momentum_quadrature(int N, double* x, double* W) {
  if (!x || !W) return fail(SBZ_ERR_ARG, "null output");
  const int r = sbz::momentum_quadrature(N, x, W);
  return r == SBZ_OK ? SBZ_OK : fail(r, "N must be in 1..8");
}

int sbz_problem_create(const sbz_model* m, const sbz_params* p, int n_cosmo, const sbz_opts* o, sbz_problem** out) {
  if (!m || !p || !out || n_cosmo < 1) return fail(SBZ_ERR_ARG, "sbz_problem_create: bad arguments");
  *out = nullptr;
  auto* pb = new sbz_problem();
  pb->model = *m;
  if (o) pb->opts = *o; else sbz_default_opts(&pb->opts);
  if (pb->opts.table_points < 16) pb->opts.table_points = 8192;
  pb->ncosmo = n_cosmo;
  pb->params.assign(p, p + n_cosmo);
  int r = sbz::build_model(*m, pb->M, pb->comps);
  if (r != SBZ_OK) { delete pb; return fail(r, "unsupported model (lmax >= 3, 0 <= nx_h <= 8)"); }
  if ((pb->M.n + 31) / 32 > 6) { delete pb; return fail(SBZ_ERR_ARG, "perturbation state larger than 192 unknowns"); }
  *out = pb;
  return SBZ_OK;
}

int sbz_problem_set_params(sbz_problem* pb, const sbz_params* p, int n_cosmo) {
  if (!pb || !p || n_cosmo < 1) return fail(SBZ_ERR_ARG, "sbz_problem_set_params: bad arguments");
  if (pb->stream && cudaStreamSynchronize(pb->stream) != cudaSuccess) return fail(SBZ_ERR_CUDA, "stream");
  pb->params.assign(p, p + n_cosmo);
  pb->ncosmo = n_cosmo;
  pb->bgs.clear(); pb->bg_status.clear(); pb->cds.clear();
  pb->bg_done = false;
  pb->tables_uploaded = false;
  return SBZ_OK;
}

// Device resources are created on first use, so the host stages (background, tables) run
// without a GPU.
static int ensure_device(sbz_problem* pb) {
  if (pb->stream) return SBZ_OK;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&pb->num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return fail(SBZ_ERR_CUDA, "no CUDA device");
  if (cudaStreamCreateWithFlags(&pb->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(SBZ_ERR_CUDA, "stream");
  return SBZ_OK;
}

static int upload_tables(sbz_problem* pb);

static int ensure_events(sbz_problem* pb) {
  if (pb->ev[0]) return SBZ_OK;
  for (auto& e : pb->ev) if (cudaEventCreate(&e) != cudaSuccess) return fail(SBZ_ERR_CUDA, "event");
  return SBZ_OK;
}

int sbz_problem_set_stream(sbz_problem* pb, void* stream) {
  if (!pb) return fail(SBZ_ERR_ARG, "null problem");
  int r = ensure_device(pb);
  if (r != SBZ_OK) return r;
  if (pb->own_stream && pb->stream) cudaStreamDestroy(pb->stream);
  pb->stream = stream ? (cudaStream_t)stream : nullptr;
  pb->own_stream = false;
  if (!stream) { pb->own_stream = true; if (cudaStreamCreateWithFlags(&pb->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(SBZ_ERR_CUDA, "stream"); }
  return SBZ_OK;
}

int sbz_problem_timings(const sbz_problem* pb, double* ms8) {
  if (!pb || !ms8) return fail(SBZ_ERR_ARG, "null argument");
  for (int i = 0; i < 8; ++i) ms8[i] = pb->timings[i];
  return SBZ_OK;
}

void sbz_problem_destroy(sbz_problem* pb) {
  if (!pb) return;
  if (pb->stream) cudaStreamSynchronize(pb->stream);
  for (DevBuf* b : {&pb->d_model, &pb->d_comps, &pb->d_cosmos, &pb->d_tables, &pb->d_counter, &pb->d_k, &pb->d_ti,
                    &pb->d_cosmo, &pb->d_order, &pb->d_taus, &pb->d_out, &pb->d_status, &pb->d_steps})
    b->release();
  for (DevBuf* b : {&pb->c_y, &pb->c_yf, &pb->c_iv, &pb->c_cp, &pb->c_id, &pb->c_z, &pb->c_Sf, &pb->c_Sp, &pb->c_ks, &pb->c_ls,
                    &pb->c_Th, &pb->c_Thp, &pb->c_P0, &pb->c_cz, &pb->c_cl, &pb->c_pa, &pb->c_pb, &pb->c_src, &pb->c_M, &pb->c_chi,
                    &pb->c_w, &pb->c_taus, &pb->c_kf, &pb->t_cos, &pb->t_knots, &pb->t_koff, &pb->t_nknot, &pb->t_kap, &pb->t_tau,
                    &pb->t_ok})
    b->release();
  for (auto& e : pb->ev) if (e) cudaEventDestroy(e);
  if (pb->stream && pb->own_stream) cudaStreamDestroy(pb->stream);
  delete pb;
}

int sbz_problem_nstate(const sbz_problem* pb) { return pb ? pb->M.n : 0; }

int sbz_solve_bg(sbz_problem* pb, double* tau0, double* kappa0, double* taurec, int* status) {
  if (!pb) return fail(SBZ_ERR_ARG, "null problem");
  const int nc = pb->ncosmo;
  pb->bgs.assign(nc, sbz::Background{});
  pb->bg_status.assign(nc, 0);
  pb->cds.assign(nc, sbz::CosmoDesc{});
  const int ntab = pb->opts.table_points;
  std::vector<int> cst(nc, SBZ_OK);
#pragma omp parallel for schedule(dynamic, 1) if (nc > 1)
  for (int c = 0; c < nc; ++c) {
    sbz::Background& B = pb->bgs[c];
    sbz_opts bo = pb->opts;
    bo.maxiters = 100000;  // solvebg keeps its own iteration cap; opts.maxiters applies to the modes
    int st = sbz::background_solve(B, pb->params[c], pb->model, bo);
    if (st == SBZ_OK) {
      sbz::background_table_grid(B, ntab);  // node values: on the device at upload (or on demand on the host)
      st = sbz::build_cosmo(B, pb->M, pb->model, pb->cds[c]);
    }
    pb->bg_status[c] = st;
  }
  for (int c = 0; c < nc; ++c) {
    const sbz::Background& B = pb->bgs[c];
    if (tau0) tau0[c] = pb->bg_status[c] == SBZ_OK ? B.tau0 : NAN;
    if (kappa0) kappa0[c] = pb->bg_status[c] == SBZ_OK ? B.kappa0 : NAN;
    if (taurec) taurec[c] = pb->bg_status[c] == SBZ_OK ? B.taurec : NAN;
    if (status) status[c] = pb->bg_status[c];
  }
  pb->tables_uploaded = false;
  pb->bg_done = true;
  return SBZ_OK;
}


static int upload_tables(sbz_problem* pb) {
  if (pb->tables_uploaded) return SBZ_OK;
  int r = ensure_device(pb);
  if (r != SBZ_OK) return r;
  const int nc = pb->ncosmo;
  const int ntab = pb->opts.table_points;
  // descriptors, then the tables built on the device from each cosmology's knots and node times
  // (failed cosmologies get a flat dummy table)
  pb->table_stride = (int64_t)ntab * sbz::kNodeStride;
  std::vector<sbz::Cosmo> cos(nc);
  std::vector<int> koff(nc, 0), nknot(nc, 0), ok(nc, 0);
  std::vector<double> kap(nc, 0.0), ttau((size_t)nc * ntab, 0.0);
  std::vector<sbz::BgKnot> knots;
  for (int c = 0; c < nc; ++c) {
    const sbz::Background& B = pb->bgs[c];
    if (pb->bg_status[c] != SBZ_OK) {
      sbz::CosmoDesc& D = pb->cds[c];
      std::memset(&D, 0, sizeof D);
      D.tau_start = D.tau0 = NAN; D.ntab = ntab; D.idlnt = 1; D.idlntf = 1;
      continue;
    }
    cos[c] = B.P; kap[c] = B.kappa0; ok[c] = 1;
    koff[c] = (int)knots.size(); nknot[c] = (int)B.knots.size();
    knots.insert(knots.end(), B.knots.begin(), B.knots.end());
    std::memcpy(&ttau[(size_t)c * ntab], B.tabtau.data(), sizeof(double) * ntab);
  }
  if (knots.empty()) knots.resize(1);
  SBZ_CUDA(pb->t_cos.ensure(sizeof(sbz::Cosmo) * nc));
  SBZ_CUDA(pb->t_knots.ensure(sizeof(sbz::BgKnot) * knots.size()));
  SBZ_CUDA(pb->t_koff.ensure(sizeof(int) * nc));
  SBZ_CUDA(pb->t_nknot.ensure(sizeof(int) * nc));
  SBZ_CUDA(pb->t_ok.ensure(sizeof(int) * nc));
  SBZ_CUDA(pb->t_kap.ensure(sizeof(double) * nc));
  SBZ_CUDA(pb->t_tau.ensure(sizeof(double) * ttau.size()));
  SBZ_CUDA(pb->d_tables.ensure(sizeof(double) * (size_t)nc * pb->table_stride));
  SBZ_CUDA(cudaMemcpyAsync(pb->t_cos.p, cos.data(), sizeof(sbz::Cosmo) * nc, cudaMemcpyHostToDevice, pb->stream));
  SBZ_CUDA(cudaMemcpyAsync(pb->t_knots.p, knots.data(), sizeof(sbz::BgKnot) * knots.size(), cudaMemcpyHostToDevice, pb->stream));
  SBZ_CUDA(cudaMemcpyAsync(pb->t_koff.p, koff.data(), sizeof(int) * nc, cudaMemcpyHostToDevice, pb->stream));
  SBZ_CUDA(cudaMemcpyAsync(pb->t_nknot.p, nknot.data(), sizeof(int) * nc, cudaMemcpyHostToDevice, pb->stream));
  SBZ_CUDA(cudaMemcpyAsync(pb->t_ok.p, ok.data(), sizeof(int) * nc, cudaMemcpyHostToDevice, pb->stream));
  SBZ_CUDA(cudaMemcpyAsync(pb->t_kap.p, kap.data(), sizeof(double) * nc, cudaMemcpyHostToDevice, pb->stream));
  SBZ_CUDA(cudaMemcpyAsync(pb->t_tau.p, ttau.data(), sizeof(double) * ttau.size(), cudaMemcpyHostToDevice, pb->stream));
  if (sbz::table_build_launch(ntab, nc, pb->t_cos.as<sbz::Cosmo>(), pb->t_knots.as<sbz::BgKnot>(), pb->t_koff.as<int>(),
                              pb->t_nknot.as<int>(), pb->t_kap.as<double>(), pb->t_tau.as<double>(), pb->t_ok.as<int>(),
                              pb->d_tables.as<double>(), pb->table_stride, pb->stream) != SBZ_OK)
    return fail(SBZ_ERR_CUDA, "coefficient table build");
  SBZ_CUDA(pb->d_model.ensure(sizeof(sbz::ModelDesc)));
  SBZ_CUDA(pb->d_comps.ensure(sizeof(sbz::CompDesc) * pb->comps.size()));
  SBZ_CUDA(pb->d_cosmos.ensure(sizeof(sbz::CosmoDesc) * nc));
  SBZ_CUDA(pb->d_counter.ensure(sizeof(unsigned)));
  SBZ_CUDA(cudaMemcpyAsync(pb->d_model.p, &pb->M, sizeof(sbz::ModelDesc), cudaMemcpyHostToDevice, pb->stream));
  SBZ_CUDA(cudaMemcpyAsync(pb->d_comps.p, pb->comps.data(), sizeof(sbz::CompDesc) * pb->comps.size(), cudaMemcpyHostToDevice, pb->stream));
  SBZ_CUDA(cudaMemcpyAsync(pb->d_cosmos.p, pb->cds.data(), sizeof(sbz::CosmoDesc) * nc, cudaMemcpyHostToDevice, pb->stream));
  SBZ_CUDA(cudaStreamSynchronize(pb->stream));
  pb->tables_uploaded = true;
  return SBZ_OK;
}

int sbz_bg_knots(const sbz_problem* pb, int cosmo, int cap, double* tau, double* y5) {
  if (!pb || !pb->bg_done || cosmo < 0 || cosmo >= pb->ncosmo) return fail(SBZ_ERR_STATE, "background not solved");
  const auto& K = pb->bgs[cosmo].knots;
  const int n = (int)K.size();
  for (int i = 0; i < n && i < cap; ++i) {
    if (tau) tau[i] = K[i].t;
    if (y5) for (int j = 0; j < 5; ++j) y5[5 * i + j] = K[i].y[j];
  }
  return n;
}

int sbz_bg_eval(const sbz_problem* pb, int cosmo, int n, const double* tau, double* out9) {
  if (!pb || !pb->bg_done || cosmo < 0 || cosmo >= pb->ncosmo || pb->bg_status[cosmo] != SBZ_OK) return fail(SBZ_ERR_STATE, "background not solved");
  for (int i = 0; i < n; ++i) sbz::background_eval(pb->bgs[cosmo], tau[i], out9 + 9 * i);
  return SBZ_OK;
}

int sbz_bg_coefficients(const sbz_problem* pb, int cosmo, int n, const double* tau, double* out7) {
  if (!pb || !pb->bg_done || cosmo < 0 || cosmo >= pb->ncosmo || pb->bg_status[cosmo] != SBZ_OK) return fail(SBZ_ERR_STATE, "background not solved");
  // The kernels' table is built on the device.  The host copy of its values is made on first use:
  // downloaded from the device when there is one (bit-identical to what the kernels read),
  // otherwise built on the host from the same table_node code.
  sbz_problem* pm = const_cast<sbz_problem*>(pb);
  sbz::Background& B = pm->bgs[cosmo];
  if (B.tab.empty()) {
    int dev = 0;
    bool got = false;
    if (cudaGetDevice(&dev) == cudaSuccess && upload_tables(pm) == SBZ_OK) {
      std::vector<double> nodes((size_t)pm->table_stride);
      if (cudaMemcpyAsync(nodes.data(), pm->d_tables.as<double>() + (size_t)cosmo * pm->table_stride, sizeof(double) * nodes.size(),
                          cudaMemcpyDeviceToHost, pm->stream) == cudaSuccess &&
          cudaStreamSynchronize(pm->stream) == cudaSuccess) {
        B.tab.resize((size_t)B.ntab * sbz::kTabStride);
        for (int g = 0; g < B.ntab; ++g)
          std::memcpy(&B.tab[(size_t)g * sbz::kTabStride], &nodes[(size_t)g * sbz::kNodeStride + 2], sizeof(double) * sbz::kTabStride);
        got = true;
      }
    }
    if (!got) { cudaGetLastError(); sbz::background_table_values(B); }
  }
  for (int i = 0; i < n; ++i) sbz::table_eval(B, tau[i], out7 + 7 * i);
  return SBZ_OK;
}

static int pt_run(sbz_problem* pb, int nk, const int* d_cosmo, const double* d_ks, const double* d_ti, const int* d_order,
                  int ntau, const double* d_taus, int output, double* d_out, int* d_status, int64_t* d_steps) {
  sbz::PtArgs A{};
  A.model = pb->d_model.as<sbz::ModelDesc>();
  A.comps = pb->d_comps.as<sbz::CompDesc>();
  A.model_n = pb->M.n;
  A.cosmos = pb->d_cosmos.as<sbz::CosmoDesc>();
  A.tables = pb->d_tables.as<double>();
  A.table_stride = pb->table_stride;
  A.item_cosmo = d_cosmo; A.item_k = d_ks; A.item_tau_ini = d_ti; A.order = d_order; A.nitems = nk;
  A.taus = ntau > 0 ? d_taus : nullptr; A.ntau = ntau;
  A.output = output; A.out = d_out; A.status = d_status; A.steps = d_steps;
  A.rtol = pb->opts.pt_rtol; A.atol = pb->opts.pt_atol; A.maxiters = pb->opts.maxiters;
  A.refine = pb->opts.precision == SBZ_MIXED ? std::max(0, pb->opts.refine_iters) : 0;
  A.refine_skip = (float)pb->opts.refine_skip;
  A.counter = pb->d_counter.as<unsigned>();
  SBZ_CUDA(cudaMemsetAsync(A.counter, 0, sizeof(unsigned), pb->stream));
  const int r = sbz::pt_launch(A, pb->opts.precision, pb->opts.warps_per_block, pb->opts.warps_per_mode, pb->opts.blocks_per_sm, pb->num_sms, pb->stream);
  if (r != SBZ_OK) return fail(r, std::string("perturbation kernel launch: ") + cudaGetErrorString(cudaGetLastError()));
  return SBZ_OK;
}

static bool check_pt_args(sbz_problem* pb, int nk, int ntau, int output) {
  if (!pb || !pb->bg_done) { fail(SBZ_ERR_STATE, "call sbz_solve_bg first"); return false; }
  if (upload_tables(pb) != SBZ_OK) return false;
  if (nk < 0 || ntau < 0 || output < SBZ_OUT_SOURCES || output > SBZ_OUT_FACTORS) { fail(SBZ_ERR_ARG, "bad sizes or output"); return false; }
  if (output != SBZ_OUT_DELTA_M && ntau == 0) { fail(SBZ_ERR_ARG, "saved times required"); return false; }
  return true;
}

int sbz_pt_rhs(sbz_problem* pb, int nk, const int* cosmo, const double* ks, const double* taus, const double* y,
               double* f, double* dfdtau) {
  if (!pb || !pb->bg_done) return fail(SBZ_ERR_STATE, "call sbz_solve_bg first");
  if (nk <= 0 || !ks || !taus || !y || !f || !dfdtau) return fail(SBZ_ERR_ARG, "bad arguments");
  int r = upload_tables(pb);
  if (r != SBZ_OK) return r;
  const int n = pb->M.n;
  std::vector<int> cos(nk, 0);
  if (cosmo) std::copy(cosmo, cosmo + nk, cos.begin());
  for (int i = 0; i < nk; ++i) if (cos[i] < 0 || cos[i] >= pb->ncosmo || pb->bg_status[cos[i]] != SBZ_OK) return fail(SBZ_ERR_ARG, "bad cosmology");
  for (int i = 0; i < nk; ++i) if (!(taus[i] >= pb->bgs[cos[i]].tau_start && taus[i] <= pb->bgs[cos[i]].tau0)) return fail(SBZ_ERR_ARG, "tau outside the background span");
  double *d_k, *d_t, *d_y, *d_f, *d_ft; int* d_c;
  const size_t ny = sizeof(double) * (size_t)nk * n;
  SBZ_CUDA(cudaMalloc(&d_k, sizeof(double) * nk)); SBZ_CUDA(cudaMalloc(&d_t, sizeof(double) * nk));
  SBZ_CUDA(cudaMalloc(&d_c, sizeof(int) * nk)); SBZ_CUDA(cudaMalloc(&d_y, ny));
  SBZ_CUDA(cudaMalloc(&d_f, ny)); SBZ_CUDA(cudaMalloc(&d_ft, ny));
  SBZ_CUDA(cudaMemcpy(d_k, ks, sizeof(double) * nk, cudaMemcpyHostToDevice));
  SBZ_CUDA(cudaMemcpy(d_t, taus, sizeof(double) * nk, cudaMemcpyHostToDevice));
  SBZ_CUDA(cudaMemcpy(d_c, cos.data(), sizeof(int) * nk, cudaMemcpyHostToDevice));
  SBZ_CUDA(cudaMemcpy(d_y, y, ny, cudaMemcpyHostToDevice));
  sbz::PtArgs A{};
  A.model = pb->d_model.as<sbz::ModelDesc>(); A.comps = pb->d_comps.as<sbz::CompDesc>(); A.model_n = n;
  A.cosmos = pb->d_cosmos.as<sbz::CosmoDesc>(); A.tables = pb->d_tables.as<double>(); A.table_stride = pb->table_stride;
  A.item_cosmo = d_c; A.item_k = d_k; A.nitems = nk;
  r = sbz::rhs_launch(A, d_y, d_t, d_f, d_ft, pb->stream);
  if (r == SBZ_OK) {
    SBZ_CUDA(cudaStreamSynchronize(pb->stream));
    SBZ_CUDA(cudaMemcpy(f, d_f, ny, cudaMemcpyDeviceToHost));
    SBZ_CUDA(cudaMemcpy(dfdtau, d_ft, ny, cudaMemcpyDeviceToHost));
  }
  for (void* p : {(void*)d_k, (void*)d_t, (void*)d_c, (void*)d_y, (void*)d_f, (void*)d_ft}) cudaFree(p);
  return r == SBZ_OK ? SBZ_OK : fail(r, "rhs kernel");
}

int sbz_solve_pt_device(sbz_problem* pb, int nk, const int* cosmo, const double* ks, const double* tau_ini, int ntau,
                        const double* taus, int output, double* out, int* status, int64_t* steps) {
  if (!check_pt_args(pb, nk, ntau, output)) return SBZ_ERR_ARG;
  if (nk == 0) return SBZ_OK;
  return pt_run(pb, nk, cosmo, ks, tau_ini, nullptr, ntau, taus, output, out, status, steps);
}

int sbz_solve_pt(sbz_problem* pb, int nk, const int* cosmo, const double* ks, const double* tau_ini, int ntau,
                 const double* taus, int output, double* out, int* status, int64_t* steps) {
  if (!check_pt_args(pb, nk, ntau, output)) return SBZ_ERR_ARG;
  if (nk == 0) return SBZ_OK;
  for (int i = 0; i < nk; ++i) {
    const int c = cosmo ? cosmo[i] : 0;
    if (c < 0 || c >= pb->ncosmo) return fail(SBZ_ERR_ARG, "cosmology index out of range");
  }
  const int n = pb->M.n;
  const size_t nout = output == SBZ_OUT_DELTA_M ? (size_t)nk : output == SBZ_OUT_SOURCES ? (size_t)nk * ntau * 3
                      : output == SBZ_OUT_SOURCES4 ? (size_t)nk * ntau * 4 : output == SBZ_OUT_FACTORS ? (size_t)nk * ntau * 7
                      : (size_t)nk * ntau * n;
  // longest-first work order: high-k modes take the most steps
  std::vector<int> order(nk);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return ks[a] > ks[b]; });
  std::vector<int> cos(nk, 0);
  if (cosmo) std::copy(cosmo, cosmo + nk, cos.begin());
  SBZ_CUDA(pb->d_k.ensure(sizeof(double) * nk));
  SBZ_CUDA(pb->d_ti.ensure(sizeof(double) * nk));
  SBZ_CUDA(pb->d_cosmo.ensure(sizeof(int) * nk));
  SBZ_CUDA(pb->d_order.ensure(sizeof(int) * nk));
  SBZ_CUDA(pb->d_taus.ensure(sizeof(double) * std::max<size_t>(1, (size_t)ntau * pb->ncosmo)));
  SBZ_CUDA(pb->d_out.ensure(sizeof(double) * nout));
  SBZ_CUDA(pb->d_status.ensure(sizeof(int) * nk));
  SBZ_CUDA(pb->d_steps.ensure(sizeof(int64_t) * 2 * nk));
  cudaStream_t st = pb->stream;
  SBZ_CUDA(cudaMemcpyAsync(pb->d_k.p, ks, sizeof(double) * nk, cudaMemcpyHostToDevice, st));
  SBZ_CUDA(cudaMemcpyAsync(pb->d_ti.p, tau_ini, sizeof(double) * nk, cudaMemcpyHostToDevice, st));
  SBZ_CUDA(cudaMemcpyAsync(pb->d_cosmo.p, cos.data(), sizeof(int) * nk, cudaMemcpyHostToDevice, st));
  SBZ_CUDA(cudaMemcpyAsync(pb->d_order.p, order.data(), sizeof(int) * nk, cudaMemcpyHostToDevice, st));
  if (ntau > 0) SBZ_CUDA(cudaMemcpyAsync(pb->d_taus.p, taus, sizeof(double) * ntau * pb->ncosmo, cudaMemcpyHostToDevice, st));
  int r = pt_run(pb, nk, pb->d_cosmo.as<int>(), pb->d_k.as<double>(), pb->d_ti.as<double>(), pb->d_order.as<int>(), ntau,
                 pb->d_taus.as<double>(), output, pb->d_out.as<double>(), pb->d_status.as<int>(), pb->d_steps.as<int64_t>());
  if (r != SBZ_OK) return r;
  if (out) SBZ_CUDA(cudaMemcpyAsync(out, pb->d_out.p, sizeof(double) * nout, cudaMemcpyDeviceToHost, st));
  if (status) SBZ_CUDA(cudaMemcpyAsync(status, pb->d_status.p, sizeof(int) * nk, cudaMemcpyDeviceToHost, st));
  if (steps) SBZ_CUDA(cudaMemcpyAsync(steps, pb->d_steps.p, sizeof(int64_t) * 2 * nk, cudaMemcpyDeviceToHost, st));
  SBZ_CUDA(cudaStreamSynchronize(st));
  return SBZ_OK;
}

int sbz_autotune_pt(sbz_problem* pb, int nk, const int* cosmo, const double* ks, const double* tau_ini, int ntau,
                    const double* taus, int output, int* best, double* ms) {
  if (!check_pt_args(pb, nk, ntau, output)) return SBZ_ERR_ARG;
  if (nk <= 0 || !ks || !tau_ini) return fail(SBZ_ERR_ARG, "sbz_autotune_pt: bad arguments");
  // stratified sample in k (every m-th mode of the k-sorted list): large batches are timed on an
  // eighth of their modes, small ones in full, so the sample stays in the same regime (tail-bound
  // or throughput-bound) as the workload
  std::vector<int> byk(nk);
  std::iota(byk.begin(), byk.end(), 0);
  std::stable_sort(byk.begin(), byk.end(), [&](int a, int b) { return ks[a] > ks[b]; });
  const int m = nk > 2048 ? 8 : 1;
  std::vector<int> sc, order;
  std::vector<double> sk, st;
  for (int i = 0; i < nk; i += m) {
    const int j = byk[i];
    const int c = cosmo ? cosmo[j] : 0;
    if (c < 0 || c >= pb->ncosmo) return fail(SBZ_ERR_ARG, "cosmology index out of range");
    sk.push_back(ks[j]); st.push_back(tau_ini[j]); sc.push_back(c); order.push_back((int)order.size());
  }
  const int ns = (int)sk.size(), n = pb->M.n;
  const size_t nout = output == SBZ_OUT_DELTA_M ? (size_t)ns : output == SBZ_OUT_SOURCES ? (size_t)ns * ntau * 3
                      : output == SBZ_OUT_SOURCES4 ? (size_t)ns * ntau * 4 : output == SBZ_OUT_FACTORS ? (size_t)ns * ntau * 7
                      : (size_t)ns * ntau * n;
  cudaStream_t s = pb->stream;
  SBZ_CUDA(pb->d_k.ensure(sizeof(double) * ns));
  SBZ_CUDA(pb->d_ti.ensure(sizeof(double) * ns));
  SBZ_CUDA(pb->d_cosmo.ensure(sizeof(int) * ns));
  SBZ_CUDA(pb->d_order.ensure(sizeof(int) * ns));
  SBZ_CUDA(pb->d_taus.ensure(sizeof(double) * std::max<size_t>(1, (size_t)ntau * pb->ncosmo)));
  SBZ_CUDA(pb->d_out.ensure(sizeof(double) * nout));
  SBZ_CUDA(pb->d_status.ensure(sizeof(int) * ns));
  SBZ_CUDA(pb->d_steps.ensure(sizeof(int64_t) * 2 * ns));
  SBZ_CUDA(cudaMemcpyAsync(pb->d_k.p, sk.data(), sizeof(double) * ns, cudaMemcpyHostToDevice, s));
  SBZ_CUDA(cudaMemcpyAsync(pb->d_ti.p, st.data(), sizeof(double) * ns, cudaMemcpyHostToDevice, s));
  SBZ_CUDA(cudaMemcpyAsync(pb->d_cosmo.p, sc.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, s));
  SBZ_CUDA(cudaMemcpyAsync(pb->d_order.p, order.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, s));
  if (ntau > 0) SBZ_CUDA(cudaMemcpyAsync(pb->d_taus.p, taus, sizeof(double) * ntau * pb->ncosmo, cudaMemcpyHostToDevice, s));
  int r;
  if ((r = ensure_events(pb)) != SBZ_OK) return r;
  const int cand[SBZ_TUNE_CANDIDATES][2] = {{1, 0}, {2, 0}, {2, 2}, {4, 1}, {4, 2}, {4, 3}, {8, 1}};
  const int keep_nw = pb->opts.warps_per_mode, keep_bps = pb->opts.blocks_per_sm;
  double best_ms = 1e300;
  int bi = 0;
  for (int c = 0; c < SBZ_TUNE_CANDIDATES; ++c) {
    pb->opts.warps_per_mode = cand[c][0];
    pb->opts.blocks_per_sm = cand[c][1];
    SBZ_CUDA(cudaEventRecord(pb->ev[8], s));
    r = pt_run(pb, ns, pb->d_cosmo.as<int>(), pb->d_k.as<double>(), pb->d_ti.as<double>(), pb->d_order.as<int>(), ntau,
               pb->d_taus.as<double>(), output, pb->d_out.as<double>(), pb->d_status.as<int>(), pb->d_steps.as<int64_t>());
    if (r != SBZ_OK) { pb->opts.warps_per_mode = keep_nw; pb->opts.blocks_per_sm = keep_bps; return r; }
    SBZ_CUDA(cudaEventRecord(pb->ev[9], s));
    SBZ_CUDA(cudaEventSynchronize(pb->ev[9]));
    float t = 0;
    cudaEventElapsedTime(&t, pb->ev[8], pb->ev[9]);
    if (ms) ms[c] = t;
    if (t < best_ms) { best_ms = t; bi = c; }
  }
  pb->opts.warps_per_mode = cand[bi][0];
  pb->opts.blocks_per_sm = cand[bi][1];
  if (best) { best[0] = cand[bi][0]; best[1] = cand[bi][1]; }
  return SBZ_OK;
}

int sbz_spectrum_primordial(const sbz_problem* pb, int cosmo, int nk, const double* ks, double* P0) {
  if (!pb || cosmo < 0 || cosmo >= pb->ncosmo) return fail(SBZ_ERR_ARG, "bad cosmology");
  sbz::Cosmo P;
  sbz::cosmo_derive(P, pb->params[cosmo], pb->model);
  for (int i = 0; i < nk; ++i) P0[i] = 2 * M_PI * M_PI * P.As / (ks[i] * ks[i] * ks[i]) * std::pow(ks[i] / P.kpivot, P.ns - 1);
  return SBZ_OK;
}

int sbz_spectrum_matter(sbz_problem* pb, int nk, const int* cosmo, const double* ks, double ktau_ini, double tau_ini_max,
                        double* Pk, int* status) {
  if (!pb || !Pk) return fail(SBZ_ERR_ARG, "null argument");
  std::vector<double> ti(nk), dm(nk);
  for (int i = 0; i < nk; ++i) ti[i] = std::min(ktau_ini / ks[i], tau_ini_max);
  int r = sbz_solve_pt(pb, nk, cosmo, ks, ti.data(), 0, nullptr, SBZ_OUT_DELTA_M, dm.data(), status, nullptr);
  if (r != SBZ_OK) return r;
  for (int i = 0; i < nk; ++i) {
    const int c = cosmo ? cosmo[i] : 0;
    double P0;
    sbz_spectrum_primordial(pb, c, 1, ks + i, &P0);
    Pk[i] = P0 * dm[i] * dm[i];
  }
  return SBZ_OK;
}

static int spectrum_cmb_impl(sbz_problem* pb, int cosmo, const sbz_bessel* jl, int nc, const double* ks_coarse, const double* yc,
                             const double* wc, int interp, int ntau, const double* taus, const double* coarse_sources, int nf,
                             const double* ks_fine, const double* yf, int npair, const int* pair_a, const int* pair_b, int l_limber,
                             double* out_cl, int* status);

int sbz_spectrum_cmb(sbz_problem* pb, int cosmo, const sbz_bessel* jl, int nc, const double* ks_coarse, const double* yc,
                     const double* wc, int interp, int ntau, const double* taus, int nf, const double* ks_fine, const double* yf,
                     int npair, const int* pair_a, const int* pair_b, int l_limber, double* out_cl, int* status) {
  return spectrum_cmb_impl(pb, cosmo, jl, nc, ks_coarse, yc, wc, interp, ntau, taus, nullptr, nf, ks_fine, yf, npair, pair_a, pair_b,
                           l_limber, out_cl, status);
}

int sbz_spectrum_cmb_sources(sbz_problem* pb, int cosmo, const sbz_bessel* jl, int nc, const double* ks_coarse, const double* yc,
                             const double* wc, int interp, int ntau, const double* taus, const double* sources, int nf,
                             const double* ks_fine, const double* yf, int npair, const int* pair_a, const int* pair_b, int l_limber,
                             double* out_cl) {
  if (!sources) return fail(SBZ_ERR_ARG, "null sources");
  return spectrum_cmb_impl(pb, cosmo, jl, nc, ks_coarse, yc, wc, interp, ntau, taus, sources, nf, ks_fine, yf, npair, pair_a, pair_b,
                           l_limber, out_cl, nullptr);
}

static int spectrum_cmb_impl(sbz_problem* pb, int cosmo, const sbz_bessel* jl, int nc, const double* ks_coarse, const double* yc,
                             const double* wc, int interp, int ntau, const double* taus, const double* coarse_sources, int nf,
                             const double* ks_fine, const double* yf, int npair, const int* pair_a, const int* pair_b, int l_limber,
                             double* out_cl, int* status) {
  if (!pb || !jl || !ks_coarse || !yc || !taus || !ks_fine || !yf || !pair_a || !pair_b || !out_cl) return fail(SBZ_ERR_ARG, "null argument");
  if (nc < 3 || ntau < 2 || nf < 2 || npair < 1 || cosmo < 0 || cosmo >= pb->ncosmo) return fail(SBZ_ERR_ARG, "bad sizes");
  if (interp == SBZ_KINTERP_BARYCENTRIC && !wc) return fail(SBZ_ERR_ARG, "barycentric weights required");
  if (!pb->bg_done) return fail(SBZ_ERR_STATE, "call sbz_solve_bg first");
  if (pb->bg_status[cosmo] != SBZ_OK) return fail(SBZ_ERR_STATE, "background failed for this cosmology");
  for (int q = 0; q < npair; ++q) if (pair_a[q] < 0 || pair_a[q] > 2 || pair_b[q] < 0 || pair_b[q] > 2) return fail(SBZ_ERR_ARG, "pair sources must be 0 (T), 1 (E) or 2 (psi)");
  for (int i = 1; i < nf; ++i) if (!(ks_fine[i] > ks_fine[i - 1] && yf[i] > yf[i - 1])) return fail(SBZ_ERR_ARG, "fine grid must increase");
  const double tau_span = taus[ntau - 1] - taus[0];
  if (!(jl->J.xmax >= ks_fine[nf - 1] * tau_span)) return fail(SBZ_ERR_ARG, "Bessel cache xmax < kmax * (τ0 - τ_first)");
  int r = upload_tables(pb);
  if (r != SBZ_OK) return r;
  if ((r = ensure_events(pb)) != SBZ_OK) return r;
  cudaStream_t st = pb->stream;
  const int nl = jl->J.nl;
  // which sources: T/E block (no Limber) and ψ (with Limber), as the reference does
  bool use[3] = {false, false, false};
  for (int q = 0; q < npair; ++q) { use[pair_a[q]] = true; use[pair_b[q]] = true; }
  std::vector<int> srcTE, srcP;
  int colof[3] = {-1, -1, -1};
  for (int s = 0; s < 2; ++s) if (use[s]) { colof[s] = (int)srcTE.size(); srcTE.push_back(s); }
  if (use[2]) { srcP.push_back(2); }
  const int nTE = (int)srcTE.size();
  const int ns_all = nTE + (use[2] ? 1 : 0);
  if (use[2]) colof[2] = nTE;
  // host-side grid data
  std::vector<int> iv(nf, 0);
  std::vector<double> cp, idn, Mw;
  if (interp == SBZ_KINTERP_SPLINE) {
    for (int i = 1; i < nc; ++i) if (!(yc[i] > yc[i - 1])) return fail(SBZ_ERR_ARG, "coarse y grid must increase for spline interpolation");
    std::vector<double> Y(yc, yc + nc);
    spline_factors(Y, cp, idn);
    for (int f = 0; f < nf; ++f) {
      int i = (int)(std::upper_bound(yc, yc + nc, yf[f]) - yc) - 1;
      iv[f] = std::max(0, std::min(i, nc - 2));
    }
  } else {
    Mw.assign((size_t)nf * nc, 0.0);
    for (int f = 0; f < nf; ++f) {
      double den = 0; int exact = -1;
      for (int c = 0; c < nc; ++c) { const double dy = yf[f] - yc[c]; if (dy == 0) { exact = c; break; } }
      if (exact >= 0) { Mw[(size_t)f * nc + exact] = 1; continue; }
      for (int c = 0; c < nc; ++c) { const double t = wc[c] / (yf[f] - yc[c]); Mw[(size_t)f * nc + c] = t; den += t; }
      for (int c = 0; c < nc; ++c) Mw[(size_t)f * nc + c] /= den;
    }
  }
  std::vector<double> chi(ntau), w(ntau);
  los_weights(taus, ntau, chi, w);
  std::vector<double> P0(nf);
  sbz_spectrum_primordial(pb, cosmo, nf, ks_fine, P0.data());
  std::vector<double> Xk(nf + 1), wk;
  Xk[0] = 0; for (int i = 0; i < nf; ++i) Xk[i + 1] = ks_fine[i];
  spline_integral_weights(Xk, wk);
  std::vector<double> gk(nf);  // C_l = Σ_k gk Θ_a Θ_b  (spline integral of 2/π k² P0 Θ_a Θ_b)
  for (int i = 0; i < nf; ++i) gk[i] = wk[i + 1] * (2.0 / M_PI) * ks_fine[i] * ks_fine[i] * P0[i];
  std::vector<int> cos(nc, cosmo), ord(nc);
  std::vector<double> ti(nc, pb->bgs[cosmo].tau_start);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return ks_coarse[a] > ks_coarse[b]; });
  int ilim = nl;
  for (int i = 0; i < nl; ++i) if (jl->ls[i] >= l_limber) { ilim = i; break; }
  std::vector<int> pa(npair), pbv(npair);
  for (int q = 0; q < npair; ++q) { pa[q] = colof[pair_a[q]]; pbv[q] = colof[pair_b[q]]; }

  SBZ_CUDA(cudaEventRecord(pb->ev[0], st));
  // inputs
  SBZ_CUDA(up(pb->d_k, ks_coarse, nc, st));
  SBZ_CUDA(up(pb->d_ti, ti.data(), nc, st));
  SBZ_CUDA(up(pb->d_cosmo, cos.data(), nc, st));
  SBZ_CUDA(up(pb->d_order, ord.data(), nc, st));
  SBZ_CUDA(pb->d_taus.ensure(sizeof(double) * (size_t)ntau * pb->ncosmo));
  SBZ_CUDA(cudaMemcpyAsync(pb->d_taus.as<double>() + (size_t)cosmo * ntau, taus, sizeof(double) * ntau, cudaMemcpyHostToDevice, st));
  SBZ_CUDA(up(pb->c_y, yc, nc, st));
  SBZ_CUDA(up(pb->c_yf, yf, nf, st));
  SBZ_CUDA(up(pb->c_iv, iv.data(), nf, st));
  SBZ_CUDA(up(pb->c_cp, cp.data(), cp.size(), st));
  SBZ_CUDA(up(pb->c_id, idn.data(), idn.size(), st));
  SBZ_CUDA(up(pb->c_M, Mw.data(), Mw.size(), st));
  SBZ_CUDA(up(pb->c_ks, ks_fine, nf, st));
  SBZ_CUDA(up(pb->c_chi, chi.data(), ntau, st));
  SBZ_CUDA(up(pb->c_w, w.data(), ntau, st));
  SBZ_CUDA(up(pb->c_taus, taus, ntau, st));
  SBZ_CUDA(up(pb->c_P0, P0.data(), nf, st));
  SBZ_CUDA(up(pb->c_pa, pa.data(), npair, st));
  SBZ_CUDA(up(pb->c_pb, pbv.data(), npair, st));
  std::vector<int> srcAll(srcTE); if (use[2]) srcAll.push_back(2);
  SBZ_CUDA(up(pb->c_src, srcAll.data(), srcAll.size(), st));
  SBZ_CUDA(pb->d_out.ensure(sizeof(double) * (size_t)nc * ntau * 3));
  SBZ_CUDA(pb->d_status.ensure(sizeof(int) * nc));
  SBZ_CUDA(pb->d_steps.ensure(sizeof(int64_t) * 2 * nc));
  SBZ_CUDA(cudaEventRecord(pb->ev[1], st));
  // 1. perturbation modes -> coarse sources (or the caller's coarse sources, e.g. a surrogate's)
  if (coarse_sources) {
    SBZ_CUDA(cudaMemcpyAsync(pb->d_out.p, coarse_sources, sizeof(double) * (size_t)nc * ntau * 3, cudaMemcpyHostToDevice, st));
    SBZ_CUDA(cudaMemsetAsync(pb->d_status.p, 0, sizeof(int) * nc, st));
  } else {
    sbz::PtArgs A{};
    A.model = pb->d_model.as<sbz::ModelDesc>(); A.comps = pb->d_comps.as<sbz::CompDesc>(); A.model_n = pb->M.n;
    A.cosmos = pb->d_cosmos.as<sbz::CosmoDesc>(); A.tables = pb->d_tables.as<double>(); A.table_stride = pb->table_stride;
    A.item_cosmo = pb->d_cosmo.as<int>(); A.item_k = pb->d_k.as<double>(); A.item_tau_ini = pb->d_ti.as<double>();
    A.order = pb->d_order.as<int>(); A.nitems = nc;
    A.taus = pb->d_taus.as<double>(); A.ntau = ntau; A.output = SBZ_OUT_SOURCES;
    A.out = pb->d_out.as<double>(); A.status = pb->d_status.as<int>(); A.steps = pb->d_steps.as<int64_t>();
    A.rtol = pb->opts.pt_rtol; A.atol = pb->opts.pt_atol; A.maxiters = pb->opts.maxiters;
    A.refine = pb->opts.precision == SBZ_MIXED ? std::max(0, pb->opts.refine_iters) : 0;
  A.refine_skip = (float)pb->opts.refine_skip;
    A.counter = pb->d_counter.as<unsigned>();
    SBZ_CUDA(cudaMemsetAsync(A.counter, 0, sizeof(unsigned), st));
    r = sbz::pt_launch(A, pb->opts.precision, pb->opts.warps_per_block, pb->opts.warps_per_mode, pb->opts.blocks_per_sm, pb->num_sms, st);
    if (r != SBZ_OK) return fail(r, "perturbation kernel");
    // the perturbation kernel saves the sources at taus of *this* cosmology: A.taus + cosmo*ntau
  }
  SBZ_CUDA(cudaEventRecord(pb->ev[2], st));
  // 2. interpolate to the fine k-grid; zero the last time (χ = 0, angular.jl:296)
  SBZ_CUDA(pb->c_Sf.ensure(sizeof(double) * (size_t)ntau * nf * std::max(1, nTE)));
  SBZ_CUDA(pb->c_Sp.ensure(sizeof(double) * (size_t)ntau * nf));
  SBZ_CUDA(pb->c_z.ensure(sizeof(double) * (size_t)nc * ntau * std::max(1, ns_all)));
  auto kinterp = [&](int ns, const int* d_src, double* d_out) -> int {
    if (interp == SBZ_KINTERP_SPLINE)
      return sbz::kinterp_spline_launch(nc, ntau, ns, nf, d_src, pb->d_out.as<double>(), pb->c_y.as<double>(), pb->c_yf.as<double>(),
                                        pb->c_iv.as<int>(), pb->c_cp.as<double>(), pb->c_id.as<double>(), pb->c_z.as<double>(), d_out, st);
    return sbz::kinterp_bary_launch(nc, ntau, ns, nf, d_src, pb->d_out.as<double>(), pb->c_M.as<double>(), d_out, st);
  };
  if (nTE > 0 && kinterp(nTE, pb->c_src.as<int>(), pb->c_Sf.as<double>()) != 0) return fail(SBZ_ERR_CUDA, "k-interpolation");
  if (use[2] && kinterp(1, pb->c_src.as<int>() + nTE, pb->c_Sp.as<double>()) != 0) return fail(SBZ_ERR_CUDA, "k-interpolation");
  if (nTE > 0) SBZ_CUDA(cudaMemsetAsync(pb->c_Sf.as<double>() + (size_t)(ntau - 1) * nf * nTE, 0, sizeof(double) * nf * nTE, st));
  if (use[2]) SBZ_CUDA(cudaMemsetAsync(pb->c_Sp.as<double>() + (size_t)(ntau - 1) * nf, 0, sizeof(double) * nf, st));
  SBZ_CUDA(cudaEventRecord(pb->ev[3], st));
  // 3. line-of-sight integrals and Θ scaling; gather T/E/ψ into one interleaved Θ array
  SBZ_CUDA(pb->c_Th.ensure(sizeof(double) * (size_t)nf * nl * std::max(1, nTE)));
  SBZ_CUDA(pb->c_Thp.ensure(sizeof(double) * (size_t)nf * nl));
  // mixed precision: FP32 interpolation and chunk sums (the C_l target is ~1e-4); FP64 otherwise
  const int losp = pb->opts.los_precision >= 0 ? pb->opts.los_precision : pb->opts.precision;
  auto los = losp == SBZ_MIXED && nl <= 1024 ? sbz::los_f32_launch : sbz::los_launch;
  if (nTE > 0 && los(jl->J, const_cast<sbz_bessel*>(jl)->d_ls.as<int>(), nTE, pb->c_Sf.as<double>(), pb->c_taus.as<double>(),
                     pb->c_chi.as<double>(), pb->c_w.as<double>(), ntau, nf, pb->c_ks.as<double>(), nl, pb->c_Th.as<double>(), st) != 0)
    return fail(SBZ_ERR_CUDA, "LOS kernel");
  if (use[2] && los(jl->J, const_cast<sbz_bessel*>(jl)->d_ls.as<int>(), 1, pb->c_Sp.as<double>(), pb->c_taus.as<double>(),
                    pb->c_chi.as<double>(), pb->c_w.as<double>(), ntau, nf, pb->c_ks.as<double>(), ilim, pb->c_Thp.as<double>(), st) != 0)
    return fail(SBZ_ERR_CUDA, "LOS kernel");
  if (nTE > 0 && sbz::theta_scale_launch(nf, nl, nTE, pb->c_ks.as<double>(), const_cast<sbz_bessel*>(jl)->d_ls.as<int>(),
                                         colof[0], colof[1], pb->c_Th.as<double>(), st) != 0)
    return fail(SBZ_ERR_CUDA, "theta scaling");
  SBZ_CUDA(cudaEventRecord(pb->ev[4], st));
  // 4. C_l for every requested pair (ψ pairs use the separate Θ_ψ array through an interleave copy)
  double* dTh = pb->c_Th.as<double>();
  int nsTh = nTE;
  if (use[2]) {  // interleave Θ_ψ as the last column
    SBZ_CUDA(pb->c_cl.ensure(sizeof(double) * (size_t)nf * nl * ns_all));
    SBZ_CUDA(cudaMemcpy2DAsync(pb->c_cl.p, sizeof(double) * ns_all, dTh, sizeof(double) * std::max(1, nTE), sizeof(double) * nTE,
                               (size_t)nf * nl, cudaMemcpyDeviceToDevice, st));
    SBZ_CUDA(cudaMemcpy2DAsync(pb->c_cl.as<double>() + nTE, sizeof(double) * ns_all, pb->c_Thp.p, sizeof(double), sizeof(double),
                               (size_t)nf * nl, cudaMemcpyDeviceToDevice, st));
    dTh = pb->c_cl.as<double>();
    nsTh = ns_all;
  }
  SBZ_CUDA(up(pb->c_kf, gk.data(), nf, st));
  SBZ_CUDA(pb->c_cz.ensure(sizeof(double) * (size_t)nl * npair));
  double* dCl = pb->c_cz.as<double>();
  if (sbz::cl_dot_launch(nf, pb->c_kf.as<double>(), nl, nsTh, dTh, npair, pb->c_pa.as<int>(), pb->c_pb.as<int>(), dCl, st) != 0)
    return fail(SBZ_ERR_CUDA, "C_l kernel");
  SBZ_CUDA(cudaEventRecord(pb->ev[5], st));
  SBZ_CUDA(cudaMemcpyAsync(out_cl, dCl, sizeof(double) * nl * npair, cudaMemcpyDeviceToHost, st));
  if (status) SBZ_CUDA(cudaMemcpyAsync(status, pb->d_status.p, sizeof(int) * nc, cudaMemcpyDeviceToHost, st));
  SBZ_CUDA(cudaEventRecord(pb->ev[6], st));
  SBZ_CUDA(cudaStreamSynchronize(st));
  float ms;
  const int map[6][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 4}, {4, 5}, {5, 6}};
  const int slot[6] = {T_H2D, T_PT, T_KINTERP, T_LOS, T_CL, T_D2H};
  for (int i = 0; i < 6; ++i) { cudaEventElapsedTime(&ms, pb->ev[map[i][0]], pb->ev[map[i][1]]); pb->timings[slot[i]] = ms; }
  cudaEventElapsedTime(&ms, pb->ev[0], pb->ev[6]); pb->timings[T_TOTAL] = ms;
  return SBZ_OK;
}

// ---------------------------------------------------------------------------------------------
int sbz_bessel_create(int nl, const int* ls, double xmax, double dx, int hermite, sbz_bessel** out) {
  if (!ls || nl < 1 || !out || !(xmax > 0) || !(dx > 0)) return fail(SBZ_ERR_ARG, "sbz_bessel_create: bad arguments");
  for (int i = 0; i < nl; ++i) if (ls[i] < 0 || (i && ls[i] <= ls[i - 1])) return fail(SBZ_ERR_ARG, "ls must be increasing and >= 0");
  const int N = (int)std::trunc(xmax / dx);
  if (N < 2) return fail(SBZ_ERR_ARG, "xmax/dx too small");
  auto* c = new sbz_bessel();
  c->ls.assign(ls, ls + nl);
  c->J.nl = nl; c->J.nx = N + 1; c->J.xmax = xmax; c->J.step = xmax / (N - 1); c->J.invdx = 1.0 / c->J.step; c->J.dx = dx;
  c->J.hermite = hermite ? 1 : 0;
  auto bail = [&](const char* m) { sbz_bessel_destroy(c); return fail(SBZ_ERR_CUDA, m); };
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return bail("stream");
  if (c->d_y.ensure(sizeof(double) * (size_t)c->J.nx * nl) != cudaSuccess) return bail("bessel table allocation");
  if (hermite && c->d_dy.ensure(sizeof(double) * (size_t)c->J.nx * nl) != cudaSuccess) return bail("bessel table allocation");
  if (c->d_yf2.ensure(sizeof(float2) * (size_t)c->J.nx * nl) != cudaSuccess) return bail("bessel table allocation");
  if (c->d_ls.ensure(sizeof(int) * nl) != cudaSuccess) return bail("allocation");
  c->J.y = c->d_y.as<double>(); c->J.dy = hermite ? c->d_dy.as<double>() : nullptr; c->J.yf2 = c->d_yf2.as<float2>();
  cudaMemcpyAsync(c->d_ls.p, ls, sizeof(int) * nl, cudaMemcpyHostToDevice, c->stream);
  if (sbz::bessel_build(c->J, c->d_ls.as<int>(), ls[nl - 1], c->stream) != 0) return bail("bessel kernel");
  if (sbz::bessel_f32_build(c->J, c->stream) != 0) return bail("bessel kernel");
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return bail("bessel kernel");
  *out = c;
  return SBZ_OK;
}

void sbz_bessel_destroy(sbz_bessel* c) {
  if (!c) return;
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (DevBuf* b : {&c->d_y, &c->d_dy, &c->d_yf2, &c->d_ls, &c->d_S, &c->d_taus, &c->d_chi, &c->d_w, &c->d_ks, &c->d_out}) b->release();
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

int sbz_bessel_eval(const sbz_bessel* c, int il, int n, const double* x, double* out) {
  if (!c || il < 0 || il >= c->J.nl || n < 0) return fail(SBZ_ERR_ARG, "bad arguments");
  for (int i = 0; i < n; ++i) if (!(x[i] >= 0 && x[i] <= c->J.xmax)) return fail(SBZ_ERR_ARG, "x outside the cached range");
  auto* cc = const_cast<sbz_bessel*>(c);
  SBZ_CUDA(cc->d_chi.ensure(sizeof(double) * std::max(1, n)));
  SBZ_CUDA(cc->d_out.ensure(sizeof(double) * std::max(1, n)));
  SBZ_CUDA(cudaMemcpyAsync(cc->d_chi.p, x, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
  if (sbz::bessel_eval(c->J, il, n, cc->d_chi.as<double>(), cc->d_out.as<double>(), c->stream) != 0) return fail(SBZ_ERR_CUDA, "eval kernel");
  SBZ_CUDA(cudaMemcpyAsync(out, cc->d_out.p, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
  SBZ_CUDA(cudaStreamSynchronize(c->stream));
  return SBZ_OK;
}


static int il_limber_of(const sbz_bessel* c, int l_limber) {
  int il = c->J.nl;
  for (int i = 0; i < c->J.nl; ++i) if (c->ls[i] >= l_limber) { il = i; break; }
  return il;
}

static bool los_check(const sbz_bessel* c, int nsrc, int ntau, int nk) {
  if (!c || nsrc < 1 || nsrc > 3 || ntau < 2 || nk < 0) { fail(SBZ_ERR_ARG, "bad LOS arguments (1 <= nsrc <= 3, ntau >= 2)"); return false; }
  return true;
}

int sbz_los_integrate(const sbz_bessel* c, int nsrc, const double* S, int ntau, const double* taus, int nk, const double* ks,
                      int l_limber, double* out) {
  if (!los_check(c, nsrc, ntau, nk)) return SBZ_ERR_ARG;
  for (int i = 1; i < ntau; ++i) if (!(taus[i] > taus[i - 1])) return fail(SBZ_ERR_ARG, "taus must be increasing");
  for (int i = 1; i < nk; ++i) if (!(ks[i] > ks[i - 1])) return fail(SBZ_ERR_ARG, "ks must be increasing");
  if (nk > 0 && !(c->J.xmax >= ks[nk - 1] * (taus[ntau - 1] - taus[0]))) return fail(SBZ_ERR_ARG, "Bessel cache xmax < kmax * (τ0 - τ_first)");
  const size_t ns = (size_t)ntau * nk * nsrc;
  for (size_t i = 0; i < ns; ++i) if (!std::isfinite(S[i])) return fail(SBZ_ERR_ARG, "non-finite source value");
  auto* cc = const_cast<sbz_bessel*>(c);
  std::vector<double> chi, w;
  los_weights(taus, ntau, chi, w);
  const size_t nout = (size_t)nk * c->J.nl * nsrc;
  SBZ_CUDA(cc->d_S.ensure(sizeof(double) * std::max<size_t>(1, ns)));
  SBZ_CUDA(cc->d_taus.ensure(sizeof(double) * ntau));
  SBZ_CUDA(cc->d_chi.ensure(sizeof(double) * ntau));
  SBZ_CUDA(cc->d_w.ensure(sizeof(double) * ntau));
  SBZ_CUDA(cc->d_ks.ensure(sizeof(double) * std::max(1, nk)));
  SBZ_CUDA(cc->d_out.ensure(sizeof(double) * std::max<size_t>(1, nout)));
  cudaStream_t st = c->stream;
  SBZ_CUDA(cudaMemcpyAsync(cc->d_S.p, S, sizeof(double) * ns, cudaMemcpyHostToDevice, st));
  SBZ_CUDA(cudaMemcpyAsync(cc->d_taus.p, taus, sizeof(double) * ntau, cudaMemcpyHostToDevice, st));
  SBZ_CUDA(cudaMemcpyAsync(cc->d_chi.p, chi.data(), sizeof(double) * ntau, cudaMemcpyHostToDevice, st));
  SBZ_CUDA(cudaMemcpyAsync(cc->d_w.p, w.data(), sizeof(double) * ntau, cudaMemcpyHostToDevice, st));
  SBZ_CUDA(cudaMemcpyAsync(cc->d_ks.p, ks, sizeof(double) * nk, cudaMemcpyHostToDevice, st));
  if (sbz::los_launch(c->J, cc->d_ls.as<int>(), nsrc, cc->d_S.as<double>(), cc->d_taus.as<double>(), cc->d_chi.as<double>(),
                      cc->d_w.as<double>(), ntau, nk, cc->d_ks.as<double>(), il_limber_of(c, l_limber), cc->d_out.as<double>(), st) != 0)
    return fail(SBZ_ERR_CUDA, "LOS kernel");
  SBZ_CUDA(cudaMemcpyAsync(out, cc->d_out.p, sizeof(double) * nout, cudaMemcpyDeviceToHost, st));
  SBZ_CUDA(cudaStreamSynchronize(st));
  return SBZ_OK;
}

int sbz_los_integrate_device(const sbz_bessel* c, int nsrc, const double* S, int ntau, const double* taus, int nk, const double* ks,
                             int l_limber, double* out, void* stream) {
  if (!los_check(c, nsrc, ntau, nk)) return SBZ_ERR_ARG;
  auto* cc = const_cast<sbz_bessel*>(c);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  std::vector<double> h_t(ntau), chi, w;
  SBZ_CUDA(cudaMemcpyAsync(h_t.data(), taus, sizeof(double) * ntau, cudaMemcpyDeviceToHost, st));
  SBZ_CUDA(cudaStreamSynchronize(st));
  los_weights(h_t.data(), ntau, chi, w);
  SBZ_CUDA(cc->d_chi.ensure(sizeof(double) * ntau));
  SBZ_CUDA(cc->d_w.ensure(sizeof(double) * ntau));
  SBZ_CUDA(cudaMemcpyAsync(cc->d_chi.p, chi.data(), sizeof(double) * ntau, cudaMemcpyHostToDevice, st));
  SBZ_CUDA(cudaMemcpyAsync(cc->d_w.p, w.data(), sizeof(double) * ntau, cudaMemcpyHostToDevice, st));
  if (sbz::los_launch(c->J, cc->d_ls.as<int>(), nsrc, S, taus, cc->d_chi.as<double>(), cc->d_w.as<double>(), ntau, nk, ks,
                      il_limber_of(c, l_limber), out, st) != 0)
    return fail(SBZ_ERR_CUDA, "LOS kernel");
  return SBZ_OK;
}

int sbz_cl_integrate(int nk, const double* ks, const double* P0, int nl, const double* ThA, const double* ThB, double* Cl) {
  if (nk < 2 || nl < 1 || !ks || !P0 || !ThA || !ThB || !Cl) return fail(SBZ_ERR_ARG, "sbz_cl_integrate: bad arguments");
  const int np = nk + 1;
  std::vector<double> X(np), cprime(np, 0.0), invden(np, 0.0);
  X[0] = 0;
  for (int i = 0; i < nk; ++i) X[i + 1] = ks[i];
  for (int i = 1; i < np; ++i) if (!(X[i] > X[i - 1])) return fail(SBZ_ERR_ARG, "ks must be positive and increasing");
  for (int i = 1; i <= np - 2; ++i) {
    const double h0 = X[i] - X[i - 1], h1 = X[i + 1] - X[i];
    const double den = 2 * (h0 + h1) - h0 * (i > 1 ? cprime[i - 1] : 0.0);
    invden[i] = 1.0 / den;
    cprime[i] = h1 * invden[i];
  }
  // every buffer is released on every return path, the early error returns included
  struct Owned : DevBuf {
    ~Owned() { release(); }
  } d_ks, d_P0, d_A, d_B, d_c, d_i, d_z, d_Cl;
  const size_t th = sizeof(double) * (size_t)nk * nl;
  SBZ_CUDA(d_ks.ensure(sizeof(double) * nk));
  SBZ_CUDA(d_P0.ensure(sizeof(double) * nk));
  SBZ_CUDA(d_A.ensure(th));
  SBZ_CUDA(d_B.ensure(th));
  SBZ_CUDA(d_c.ensure(sizeof(double) * np));
  SBZ_CUDA(d_i.ensure(sizeof(double) * np));
  SBZ_CUDA(d_z.ensure(sizeof(double) * (size_t)np * nl));
  SBZ_CUDA(d_Cl.ensure(sizeof(double) * nl));
  SBZ_CUDA(cudaMemcpy(d_ks.p, ks, sizeof(double) * nk, cudaMemcpyHostToDevice));
  SBZ_CUDA(cudaMemcpy(d_P0.p, P0, sizeof(double) * nk, cudaMemcpyHostToDevice));
  SBZ_CUDA(cudaMemcpy(d_A.p, ThA, th, cudaMemcpyHostToDevice));
  SBZ_CUDA(cudaMemcpy(d_B.p, ThB, th, cudaMemcpyHostToDevice));
  SBZ_CUDA(cudaMemcpy(d_c.p, cprime.data(), sizeof(double) * np, cudaMemcpyHostToDevice));
  SBZ_CUDA(cudaMemcpy(d_i.p, invden.data(), sizeof(double) * np, cudaMemcpyHostToDevice));
  int r = sbz::cl_launch(nk, d_ks.as<double>(), d_P0.as<double>(), nl, d_A.as<double>(), d_B.as<double>(), d_c.as<double>(),
                         d_i.as<double>(), d_z.as<double>(), d_Cl.as<double>(), 0);
  if (r == 0) SBZ_CUDA(cudaMemcpy(Cl, d_Cl.p, sizeof(double) * nl, cudaMemcpyDeviceToHost));
  return r == 0 ? SBZ_OK : fail(SBZ_ERR_CUDA, "C_l kernel");
}

}  // extern "C"

namespace sbz {
// error reporting for entry points defined in other translation units
int capi_fail(int code, const char* msg) { return fail(code, msg); }
}  // namespace sbz
