// Launch interface of the perturbation kernel (sbz_pt.cu).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "sbz_layout.hpp"
#include "../../include/symboltz_gb300.h"

namespace sbz {

struct PtArgs {
  const ModelDesc* model;     // device
  const CompDesc* comps;      // device, model_n entries
  int model_n;
  const CosmoDesc* cosmos;    // device, one per cosmology
  const double* tables;       // device, cosmology c at tables + c * table_stride
  int64_t table_stride;
  const int* item_cosmo;      // device, per mode (nullptr = all cosmology 0)
  const double* item_k;       // device
  const double* item_tau_ini; // device
  const int* order;           // device, processing order (nullptr = identity)
  int nitems;
  const double* taus;         // device, [c * ntau + j] (nullptr when ntau == 0)
  int ntau;
  int output;
  double* out;
  int* status;
  int64_t* steps;
  double rtol, atol;
  int64_t maxiters;
  int refine;
  float refine_skip;          // skip stages 2-6 refinement below this stage-1 correction (0: never; < 0: by launch shape)
  unsigned int* counter;      // device work-queue counter, zero before launch
};

int pt_launch(const PtArgs& A, int precision, int warps_per_block, int warps_per_mode, int blocks_per_sm, int num_sms,
              cudaStream_t stream);
int rhs_launch(const PtArgs& A, const double* y, const double* tau, double* f, double* ft, cudaStream_t st);

}  // namespace sbz
