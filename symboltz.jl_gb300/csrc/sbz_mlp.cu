// Source surrogate: dense-layer GEMM launcher (tensor maps, tile choice) and C-ABI test entry.
#include <cudaTypedefs.h>
#include <algorithm>
#include <cstdio>
#include <mutex>
#include "../../include/symboltz_gb300.h"
#include "sbz_mlp_gemm.cuh"

namespace sbz {
int capi_fail(int code, const char* msg);

namespace mlp {
namespace {

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::mutex g_mu;

bool get_encode() {
  std::lock_guard<std::mutex> lock(g_mu);
  if (g_encode) return true;
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !fn)
    return false;
  g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  return true;
}

// 2-D tensor map of a bf16 [rows][K] row-major matrix, box 64 (K) x box_rows, 128-byte swizzle
bool tmap_rows_k(CUtensorMap* tm, const void* ptr, int rows, int K, int box_rows) {
  const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)K * 2};
  const cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
  const cuuint32_t es[2] = {1, 1};
  return g_encode(tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int num_sms() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) n = 1;
  }
  return n;
}

template <int BN>
int launch(const GemmArgs& g, const void* A, const void* B, cudaStream_t st) {
  CUtensorMap ta, tb;
  if (!tmap_rows_k(&ta, A, g.M, g.K, BM) || !tmap_rows_k(&tb, B, g.N, g.K, BN)) return SBZ_ERR_CUDA;
  const size_t smem = gemm_smem_bytes<BN>();
  auto k = gemm_tn_kernel<BN>;
  static bool attr_set = false;  // set once, outside any stream capture of a later call
  if (!attr_set) {
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return SBZ_ERR_CUDA;
    attr_set = true;
  }
  const int tiles = (g.N / BN) * (g.M / BM), KT = g.K / BK;
  // weight gradients have few output tiles and a long K (the batch): split K over about two CTAs
  // per SM, at least 4 K-steps each, and add the partial tiles atomically into a zeroed output
  int splits = 1;
  if (g.epi == EPI_F32 && tiles < 2 * num_sms()) splits = std::max(1, std::min(KT / 4, 2 * num_sms() / tiles));
  if (splits > 1 && !g.accumulate) {
    for (int r = 0; r < g.M; ++r) {  // rows of the output region (ldo may exceed N)
      if (g.ldo == g.n_valid) {
        if (cudaMemsetAsync(g.out_f32, 0, sizeof(float) * (size_t)g.M * g.ldo, st) != cudaSuccess) return SBZ_ERR_CUDA;
        break;
      }
      if (cudaMemsetAsync(g.out_f32 + (size_t)r * g.ldo, 0, sizeof(float) * g.n_valid, st) != cudaSuccess) return SBZ_ERR_CUDA;
    }
  }
  const dim3 grid(g.N / BN, g.M / BM, splits);
  k<<<grid, kThreads, smem, st>>>(ta, tb, g);
  return cudaGetLastError() == cudaSuccess ? SBZ_OK : SBZ_ERR_CUDA;
}

}  // namespace

// D = A Bᵀ with the fused epilogue of g; M % 128 == 0, N % 64 == 0, K % 64 == 0, A and B 16-byte
// aligned (TMA).  The widest tile that divides N is used.
int gemm(const GemmArgs& g, const void* A, const void* B, cudaStream_t st) {
  if (g.M <= 0 || g.M % BM || g.N <= 0 || g.N % 64 || g.K <= 0 || g.K % BK) return SBZ_ERR_ARG;
  if (((uintptr_t)A | (uintptr_t)B) & 15) return SBZ_ERR_ARG;
  if (!get_encode()) return SBZ_ERR_CUDA;
  if (g.N % 256 == 0) return launch<256>(g, A, B, st);
  if (g.N % 128 == 0) return launch<128>(g, A, B, st);
  return launch<64>(g, A, B, st);
}

}  // namespace mlp
}  // namespace sbz

namespace {
unsigned* g_flag = nullptr;  // pipeline-timeout flag of the test entry (one per process)
}

extern "C" int sbz_mlp_gemm(int M, int N, int K, const void* A, const void* B, int epi, int act, const float* bias, void* out,
                            int ldo, int n_valid, int accumulate, void* z_out, const void* z_in, void* stream) {
  using namespace sbz::mlp;
  if (!A || !B || !out || epi < EPI_F32 || epi > EPI_DACT || (epi == EPI_DACT && !z_in))
    return sbz::capi_fail(SBZ_ERR_ARG, "sbz_mlp_gemm: bad arguments");
  if (!g_flag && cudaMalloc(&g_flag, sizeof(unsigned)) != cudaSuccess) return sbz::capi_fail(SBZ_ERR_CUDA, "sbz_mlp_gemm: flag");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (cudaMemsetAsync(g_flag, 0, sizeof(unsigned), st) != cudaSuccess) return sbz::capi_fail(SBZ_ERR_CUDA, "sbz_mlp_gemm: flag");
  GemmArgs g{};
  g.M = M; g.N = N; g.K = K; g.epi = epi; g.act = act; g.bias = bias;
  g.out_bf16 = static_cast<__nv_bfloat16*>(out); g.out_f32 = static_cast<float*>(out);
  g.ldo = ldo; g.n_valid = n_valid > 0 ? n_valid : N; g.accumulate = accumulate;
  g.z_out = static_cast<__nv_bfloat16*>(z_out); g.z_in = static_cast<const __nv_bfloat16*>(z_in); g.err = g_flag;
  const int r = gemm(g, A, B, st);
  if (r == SBZ_ERR_ARG) return sbz::capi_fail(r, "sbz_mlp_gemm: sizes must satisfy M%128, N%64, K%64 == 0 and 16-byte aligned operands");
  if (r != SBZ_OK) return sbz::capi_fail(r, "sbz_mlp_gemm: launch or tensor-map failure");
  unsigned flag = 0;
  if (cudaMemcpyAsync(&flag, g_flag, sizeof flag, cudaMemcpyDeviceToHost, st) != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess)
    return sbz::capi_fail(SBZ_ERR_CUDA, "sbz_mlp_gemm: kernel failed");
  if (flag) return sbz::capi_fail(SBZ_ERR_CUDA, "sbz_mlp_gemm: pipeline wait ran out");
  return SBZ_OK;
}
