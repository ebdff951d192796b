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

}  // namespace

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
  int64_t table_stride = 0;
};

struct sbz_bessel {
  sbz::BesselDev J{};
  std::vector<int> ls;
  DevBuf d_y, d_dy, d_ls;
  DevBuf d_S, d_taus, d_chi, d_w, d_ks, d_out;
  cudaStream_t stream = nullptr;
};

extern "C" {

void sbz_default_opts(sbz_opts* o) {
  o->bg_rtol = 1e-7; o->bg_atol = 1e-7; o->pt_rtol = 1e-5; o->pt_atol = 1e-5;
  o->tau_ini = 1e-6; o->tau_max = 100.0; o->maxiters = 100000;
  o->precision = SBZ_MIXED; o->refine_iters = 1; o->table_points = 8192; o->warps_per_block = 0;
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

void sbz_problem_destroy(sbz_problem* pb) {
  if (!pb) return;
  if (pb->stream) cudaStreamSynchronize(pb->stream);
  for (DevBuf* b : {&pb->d_model, &pb->d_comps, &pb->d_cosmos, &pb->d_tables, &pb->d_counter, &pb->d_k, &pb->d_ti,
                    &pb->d_cosmo, &pb->d_order, &pb->d_taus, &pb->d_out, &pb->d_status, &pb->d_steps})
    b->release();
  if (pb->stream) cudaStreamDestroy(pb->stream);
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
#pragma omp parallel for schedule(dynamic, 1)
  for (int c = 0; c < nc; ++c) {
    sbz::Background& B = pb->bgs[c];
    sbz_opts bo = pb->opts;
    bo.maxiters = 100000;  // solvebg keeps its own iteration cap; opts.maxiters applies to the modes
    int st = sbz::background_solve(B, pb->params[c], pb->model, bo);
    if (st == SBZ_OK) {
      sbz::background_table(B, ntab);
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
  // upload descriptors and tables (failed cosmologies get a flat dummy table)
  pb->table_stride = (int64_t)ntab * sbz::kNodeStride;
  std::vector<double> tabs((size_t)nc * pb->table_stride, 0.0);
  for (int c = 0; c < nc; ++c) {
    const sbz::Background& B = pb->bgs[c];
    double* T = &tabs[(size_t)c * pb->table_stride];
    if (pb->bg_status[c] != SBZ_OK) {
      sbz::CosmoDesc& D = pb->cds[c];
      std::memset(&D, 0, sizeof D);
      D.tau_start = D.tau0 = NAN; D.ntab = ntab; D.idlnt = 1;
      continue;
    }
    for (int g = 0; g < ntab; ++g) {
      double* nd = T + (size_t)g * sbz::kNodeStride;
      nd[0] = B.tabtau[g];
      nd[1] = (g + 1 < ntab) ? 1.0 / (B.tabtau[g + 1] - B.tabtau[g]) : 0.0;
      std::memcpy(nd + 2, &B.tab[(size_t)g * sbz::kTabStride], sizeof(double) * sbz::kTabStride);
    }
  }
  SBZ_CUDA(pb->d_model.ensure(sizeof(sbz::ModelDesc)));
  SBZ_CUDA(pb->d_comps.ensure(sizeof(sbz::CompDesc) * pb->comps.size()));
  SBZ_CUDA(pb->d_cosmos.ensure(sizeof(sbz::CosmoDesc) * nc));
  SBZ_CUDA(pb->d_tables.ensure(sizeof(double) * tabs.size()));
  SBZ_CUDA(pb->d_counter.ensure(sizeof(unsigned)));
  SBZ_CUDA(cudaMemcpyAsync(pb->d_model.p, &pb->M, sizeof(sbz::ModelDesc), cudaMemcpyHostToDevice, pb->stream));
  SBZ_CUDA(cudaMemcpyAsync(pb->d_comps.p, pb->comps.data(), sizeof(sbz::CompDesc) * pb->comps.size(), cudaMemcpyHostToDevice, pb->stream));
  SBZ_CUDA(cudaMemcpyAsync(pb->d_cosmos.p, pb->cds.data(), sizeof(sbz::CosmoDesc) * nc, cudaMemcpyHostToDevice, pb->stream));
  SBZ_CUDA(cudaMemcpyAsync(pb->d_tables.p, tabs.data(), sizeof(double) * tabs.size(), cudaMemcpyHostToDevice, pb->stream));
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
  const sbz::Background& B = pb->bgs[cosmo];
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
  A.counter = pb->d_counter.as<unsigned>();
  SBZ_CUDA(cudaMemsetAsync(A.counter, 0, sizeof(unsigned), pb->stream));
  const int r = sbz::pt_launch(A, pb->opts.precision, pb->opts.warps_per_block, pb->num_sms, pb->stream);
  if (r != SBZ_OK) return fail(r, std::string("perturbation kernel launch: ") + cudaGetErrorString(cudaGetLastError()));
  return SBZ_OK;
}

static bool check_pt_args(sbz_problem* pb, int nk, int ntau, int output) {
  if (!pb || !pb->bg_done) { fail(SBZ_ERR_STATE, "call sbz_solve_bg first"); return false; }
  if (upload_tables(pb) != SBZ_OK) return false;
  if (nk < 0 || ntau < 0 || output < SBZ_OUT_SOURCES || output > SBZ_OUT_STATE) { fail(SBZ_ERR_ARG, "bad sizes or output"); return false; }
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
  const size_t nout = output == SBZ_OUT_DELTA_M ? (size_t)nk : output == SBZ_OUT_SOURCES ? (size_t)nk * ntau * 3 : (size_t)nk * ntau * n;
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
  if (c->d_ls.ensure(sizeof(int) * nl) != cudaSuccess) return bail("allocation");
  c->J.y = c->d_y.as<double>(); c->J.dy = hermite ? c->d_dy.as<double>() : nullptr;
  cudaMemcpyAsync(c->d_ls.p, ls, sizeof(int) * nl, cudaMemcpyHostToDevice, c->stream);
  if (sbz::bessel_build(c->J, c->d_ls.as<int>(), ls[nl - 1], c->stream) != 0) return bail("bessel kernel");
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return bail("bessel kernel");
  *out = c;
  return SBZ_OK;
}

void sbz_bessel_destroy(sbz_bessel* c) {
  if (!c) return;
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (DevBuf* b : {&c->d_y, &c->d_dy, &c->d_ls, &c->d_S, &c->d_taus, &c->d_chi, &c->d_w, &c->d_ks, &c->d_out}) b->release();
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

static int los_weights(const double* taus, int ntau, std::vector<double>& chi, std::vector<double>& w) {
  chi.resize(ntau); w.resize(ntau);
  const double t0 = taus[ntau - 1];
  for (int i = 0; i < ntau; ++i) chi[i] = t0 - taus[i];
  w[0] = 0.5 * (taus[1] - taus[0]);
  for (int i = 1; i < ntau - 1; ++i) w[i] = 0.5 * (taus[i + 1] - taus[i - 1]);
  w[ntau - 1] = 0.5 * (taus[ntau - 1] - taus[ntau - 2]);
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
  double *d_ks, *d_P0, *d_A, *d_B, *d_c, *d_i, *d_z, *d_Cl;
  const size_t th = sizeof(double) * (size_t)nk * nl;
  SBZ_CUDA(cudaMalloc(&d_ks, sizeof(double) * nk));
  SBZ_CUDA(cudaMalloc(&d_P0, sizeof(double) * nk));
  SBZ_CUDA(cudaMalloc(&d_A, th));
  SBZ_CUDA(cudaMalloc(&d_B, th));
  SBZ_CUDA(cudaMalloc(&d_c, sizeof(double) * np));
  SBZ_CUDA(cudaMalloc(&d_i, sizeof(double) * np));
  SBZ_CUDA(cudaMalloc(&d_z, sizeof(double) * (size_t)np * nl));
  SBZ_CUDA(cudaMalloc(&d_Cl, sizeof(double) * nl));
  SBZ_CUDA(cudaMemcpy(d_ks, ks, sizeof(double) * nk, cudaMemcpyHostToDevice));
  SBZ_CUDA(cudaMemcpy(d_P0, P0, sizeof(double) * nk, cudaMemcpyHostToDevice));
  SBZ_CUDA(cudaMemcpy(d_A, ThA, th, cudaMemcpyHostToDevice));
  SBZ_CUDA(cudaMemcpy(d_B, ThB, th, cudaMemcpyHostToDevice));
  SBZ_CUDA(cudaMemcpy(d_c, cprime.data(), sizeof(double) * np, cudaMemcpyHostToDevice));
  SBZ_CUDA(cudaMemcpy(d_i, invden.data(), sizeof(double) * np, cudaMemcpyHostToDevice));
  int r = sbz::cl_launch(nk, d_ks, d_P0, nl, d_A, d_B, d_c, d_i, d_z, d_Cl, 0);
  if (r == 0) SBZ_CUDA(cudaMemcpy(Cl, d_Cl, sizeof(double) * nl, cudaMemcpyDeviceToHost));
  for (double* p : {d_ks, d_P0, d_A, d_B, d_c, d_i, d_z, d_Cl}) cudaFree(p);
  return r == 0 ? SBZ_OK : fail(SBZ_ERR_CUDA, "C_l kernel");
}

}  // extern "C"
