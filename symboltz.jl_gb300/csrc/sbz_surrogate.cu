// Source surrogate: an MLP (nin → nhidden × width, SiLU → nout) trained and evaluated with the
// project's BF16 tensor-core GEMM (sbz_mlp_gemm.cuh) and FP32 accumulation.
//
// Layout: layer l maps kin_l → nrow_l features; the input is padded to 64 columns and the output
// to 64 rows (TMA/UMMA granularity), padding weights stay zero (their gradients are zero).  Master
// weights, Adam moments and gradients are FP32 [nrow][kin]; the GEMMs read BF16 copies W [nrow][kin]
// (forward) and Wt [kin][nrow] (backward).  Activations are BF16 [batch][features], each with a
// transposed copy [features][batch] written by the same epilogue (the weight-gradient GEMMs read
// the batch as their K dimension); the last layer writes FP32 so the loss is not quantised.  A
// training step:
//   gather    X_0 (and X_0ᵀ), targets T of the step's random batch
//   forward   X_l = SiLU(X_{l-1} W_lᵀ + b_l)          (EPI_ACT, pre-activations Z_l kept, X_lᵀ)
//   loss      Y = X_L W_Lᵀ + b_L (FP32), dY = 2 (Y - T) / (batch · nout), dYᵀ, db_L = Σ_batch dY
//   backward  dZ_{l-1} = (dZ_l W_l) ⊙ SiLU'(Z_{l-1})  (EPI_DACT, dZ_{l-1}ᵀ and db_{l-1} = Σ_batch dZ_{l-1})
//             dW_l = dZ_lᵀ X_{l-1} (EPI_F32 on the transposed copies, split K)
//   Adam      one launch over every parameter: FP32 update, BF16 W and Wt refreshed.
// The step (about 20 launches) is captured once in a CUDA graph and replayed; the step counter
// and the learning rate live in device memory so the replayed graph needs no new parameters.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include "../../include/symboltz_gb300.h"
#include "sbz_mlp_gemm.cuh"

namespace sbz {
int capi_fail(int code, const char* msg);
namespace mlp {
int gemm(const GemmArgs& g, const void* A, const void* B, cudaStream_t st);
}
}  // namespace sbz

using bf16 = __nv_bfloat16;

namespace {

constexpr int kPadIn = 64, kPadOut = 64;

struct Layer {
  int kin, nrow;      // padded sizes (GEMM K and N)
  int nin, nout;      // logical sizes
  float *W, *b, *mW, *vW, *mb, *vb, *gW, *gb;  // FP32 [nrow][kin], [nrow]
  bf16 *Wh, *Wt;      // BF16 [nrow][kin], [kin][nrow]
  bool gT;            // gW holds the gradient transposed ([kin][nrow])
};

template <class T>
cudaError_t dalloc(T** p, size_t n) { return cudaMalloc(p, sizeof(T) * (n ? n : 1)); }

}  // namespace

struct sbz_surrogate {
  int nin = 0, width = 0, nhidden = 0, nout = 0, batch = 0;
  std::vector<Layer> L;
  // activations (batch rows): X[0] input, X[l] output of hidden layer l; Z[l] pre-activations
  std::vector<bf16*> X, Z, Xt, dZ, dZt;
  float* Yf = nullptr;        // [batch][64] last-layer product (before bias)
  bf16 *dY = nullptr, *dYt = nullptr;
  float* T = nullptr;         // [batch][nout] targets of the step
  double* loss = nullptr;
  unsigned* err = nullptr;
  float *dataX = nullptr, *dataY = nullptr;
  long long ndata = 0;
  long long step = 0;
  unsigned long long seed = 0;
  cudaStream_t stream = nullptr;
  long long* dstep = nullptr;  // device step counter (incremented at the start of each step)
  float* dlr = nullptr;        // device learning rate
  void* segs = nullptr;        // device table of Adam segments
  int nseg = 0;
  long long nparam_all = 0;    // padded parameter count over all segments
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
};

namespace {

// ---- kernels ---------------------------------------------------------------------------------

// Batch assembly: sample i takes data row idx = hash(step, i) mod n (uniform with replacement).
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// dstep (if not null) replaces step: the graph-captured training step reads the device counter.
// X0t (if not null) receives the transposed copy [kPadIn][batch].
__global__ void gather_batch(int batch, int nin, int nout, const float* __restrict__ dX, const float* __restrict__ dY, long long n,
                             long long step, const long long* __restrict__ dstep, unsigned long long seed, long long offset, int random,
                             bf16* __restrict__ X0, bf16* __restrict__ X0t, float* __restrict__ T) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= batch) return;
  if (dstep) step = *dstep;
  long long r;
  if (random) r = (long long)(mix64(seed ^ mix64((unsigned long long)step * 0x100000001B3ull + (unsigned long long)i)) % (unsigned long long)n);
  else r = offset + i;
  const bool live = r < n;
  bf16* x = X0 + (size_t)i * kPadIn;
  for (int j = 0; j < kPadIn; ++j) {
    const bf16 v = __float2bfloat16(live && j < nin ? dX[(size_t)r * nin + j] : 0.0f);
    x[j] = v;
    if (X0t) X0t[(size_t)j * batch + i] = v;
  }
  if (T)
    for (int j = 0; j < nout; ++j) T[(size_t)i * nout + j] = live ? dY[(size_t)r * nout + j] : 0.0f;
}

__global__ void begin_step(long long* step, double* loss) {
  ++*step;
  *loss = 0.0;
}

__global__ void set_value(float* dst, float v) { *dst = v; }

// loss and output gradient: y = Yf + b (FP32), r = y - t, dY = 2 r / (batch · nout) (BF16, padding 0);
// also dYᵀ [kPadOut][batch] and the bias gradient gb[j] += Σ_rows dY[.][j] (as rounded), when not null.
// 256 threads per block.
constexpr int kLossThreads = 256;
__global__ void __launch_bounds__(kLossThreads) loss_grad(int batch, int nout, const float* __restrict__ Yf, const float* __restrict__ b,
                                                           const float* __restrict__ T, bf16* __restrict__ dY, bf16* __restrict__ dYt,
                                                           float* __restrict__ gb, double* __restrict__ loss) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  __shared__ float cs[kLossThreads / 32][kPadOut];
  double l = 0;
  const float sc = 2.0f / ((float)batch * nout);
  for (int j = 0; j < kPadOut; ++j) {
    float g = 0.0f;
    if (i < batch && j < nout) {
      const float r = Yf[(size_t)i * kPadOut + j] + b[j] - T[(size_t)i * nout + j];
      l += (double)r * r;
      g = sc * r;
    }
    const bf16 gh = __float2bfloat16(g);
    if (i < batch) {
      dY[(size_t)i * kPadOut + j] = gh;
      if (dYt) dYt[(size_t)j * batch + i] = gh;
    }
    if (gb && j < nout) {
      float w = __bfloat162float(gh);
      for (int o = 16; o; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
      if ((threadIdx.x & 31) == 0) cs[threadIdx.x >> 5][j] = w;
    }
  }
  __shared__ double red[kLossThreads / 32];
  for (int o = 16; o; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = l;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
    atomicAdd(loss, s / ((double)batch * nout));
  }
  if (gb && threadIdx.x < nout) {
    float s = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += cs[w][threadIdx.x];
    atomicAdd(gb + threadIdx.x, s);
  }
}

// Adam over every parameter in one launch.  A segment is one layer's weights (with BF16 copies
// [nrow][kin] and [kin][nrow]; its gradient possibly transposed) or biases; `start` is its first
// index in the concatenation.  The bias corrections use the device step counter.
struct AdamSeg {
  float *p, *m, *v;
  const float* g;
  bf16 *ph, *pt;
  long long start;
  int n, gT, nrow, kin;
};

__global__ void adam_all(const AdamSeg* __restrict__ segs, int nseg, long long total, const long long* __restrict__ step,
                         const float* __restrict__ lr, float b1, float b2, float eps) {
  const float t = (float)*step, rate = *lr;
  const float c1 = 1.0f / (1.0f - exp2f(t * log2f(b1))), c2 = 1.0f / (1.0f - exp2f(t * log2f(b2)));
  int q = 0;  // a thread's indices increase, so its segment index only moves forward
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
    while (q + 1 < nseg && segs[q + 1].start <= e) ++q;
    const AdamSeg& S = segs[q];
    const int i = (int)(e - S.start);
    int r = 0, k = i;
    if (S.ph) { r = i / S.kin; k = i - r * S.kin; }
    const float gi = (S.ph && S.gT) ? S.g[(size_t)k * S.nrow + r] : S.g[i];
    const float mi = b1 * S.m[i] + (1 - b1) * gi, vi = b2 * S.v[i] + (1 - b2) * gi * gi;
    S.m[i] = mi; S.v[i] = vi;
    const float pi = S.p[i] - rate * (mi * c1) / (sqrtf(vi * c2) + eps);
    S.p[i] = pi;
    if (S.ph) { S.ph[i] = __float2bfloat16(pi); S.pt[(size_t)k * S.nrow + r] = __float2bfloat16(pi); }
  }
}

__global__ void to_bf16(int n, const float* __restrict__ p, int nrow, int kin, bf16* __restrict__ ph, bf16* __restrict__ pt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int r = i / kin, k = i - r * kin;
  ph[i] = __float2bfloat16(p[i]);
  pt[(size_t)k * nrow + r] = __float2bfloat16(p[i]);
}

__global__ void add_bias_out(int rows, int nout, const float* __restrict__ Yf, const float* __restrict__ b, float* __restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= rows * nout) return;
  const int i = t / nout, j = t - i * nout;
  out[t] = Yf[(size_t)i * kPadOut + j] + b[j];
}

// ---- host helpers ----------------------------------------------------------------------------

int F(int code, const std::string& m) { return sbz::capi_fail(code, m.c_str()); }
#define SCU(x)                                                                        \
  do {                                                                                \
    cudaError_t e_ = (x);                                                             \
    if (e_ != cudaSuccess) return F(SBZ_ERR_CUDA, std::string(#x ": ") + cudaGetErrorString(e_)); \
  } while (0)

unsigned long long splitmix(unsigned long long& s) {
  unsigned long long z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

void free_all(sbz_surrogate* s) {
  for (auto& l : s->L)
    for (void* p : {(void*)l.W, (void*)l.b, (void*)l.mW, (void*)l.vW, (void*)l.mb, (void*)l.vb, (void*)l.gW, (void*)l.gb, (void*)l.Wh,
                    (void*)l.Wt})
      if (p) cudaFree(p);
  for (auto* v : {&s->X, &s->Z, &s->Xt, &s->dZ, &s->dZt})
    for (bf16* p : *v) if (p) cudaFree(p);
  for (void* p : {(void*)s->Yf, (void*)s->dY, (void*)s->dYt, (void*)s->T, (void*)s->loss, (void*)s->err, (void*)s->dataX, (void*)s->dataY,
                  (void*)s->dstep, (void*)s->dlr, s->segs})
    if (p) cudaFree(p);
  if (s->graph_exec) cudaGraphExecDestroy(s->graph_exec);
  if (s->graph) cudaGraphDestroy(s->graph);
  if (s->stream) cudaStreamDestroy(s->stream);
}

int refresh_bf16(sbz_surrogate* s) {
  for (auto& l : s->L) {
    const int n = l.nrow * l.kin;
    to_bf16<<<(n + 255) / 256, 256, 0, s->stream>>>(n, l.W, l.nrow, l.kin, l.Wh, l.Wt);
  }
  return cudaGetLastError() == cudaSuccess ? SBZ_OK : F(SBZ_ERR_CUDA, "surrogate: weight copy");
}

int gemm(sbz_surrogate* s, int M, int N, int K, const bf16* A, const bf16* B, int epi, int act, const float* bias, void* out, int ldo,
         int n_valid, int acc, bf16* z_out, const bf16* z_in, bf16* out_t = nullptr, float* colsum = nullptr) {
  using namespace sbz::mlp;
  GemmArgs g{};
  g.M = M; g.N = N; g.K = K; g.epi = epi; g.act = act; g.bias = bias;
  g.out_bf16 = static_cast<bf16*>(out); g.out_f32 = static_cast<float*>(out); g.ldo = ldo; g.n_valid = n_valid; g.accumulate = acc;
  g.z_out = z_out; g.z_in = z_in; g.err = s->err;
  g.out_t = out_t; g.ldt = M; g.colsum = colsum;
  const int r = sbz::mlp::gemm(g, A, B, s->stream);
  return r == SBZ_OK ? SBZ_OK : F(r, "surrogate: GEMM launch");
}

// forward pass of `rows` (multiple of 128, ≤ batch) rows already in X[0]; result in Yf.  With
// `train`, the transposed activations X_lᵀ (row stride `rows`) are written for the backward pass.
int forward(sbz_surrogate* s, int rows, bool train) {
  using namespace sbz::mlp;
  const int nl = (int)s->L.size();
  for (int l = 0; l < nl - 1; ++l) {
    const Layer& y = s->L[l];
    int r = gemm(s, rows, y.nrow, y.kin, s->X[l], y.Wh, EPI_ACT, ACT_SILU, y.b, s->X[l + 1], y.nrow, y.nrow, 0, s->Z[l + 1], nullptr,
                 train ? s->Xt[l + 1] : nullptr);
    if (r) return r;
  }
  const Layer& o = s->L[nl - 1];
  return gemm(s, rows, o.nrow, o.kin, s->X[nl - 1], o.Wh, EPI_F32, ACT_NONE, nullptr, s->Yf, kPadOut, kPadOut, 0, nullptr, nullptr);
}

// backward pass after forward(train) + loss_grad (dY, dYᵀ and the output layer's gb set): weight
// gradients into gW, bias gradients accumulated into gb by the EPI_DACT epilogues
int backward(sbz_surrogate* s) {
  using namespace sbz::mlp;
  const int B = s->batch, nl = (int)s->L.size();
  // output layer: dW_Lᵀ = X_{L-1}ᵀ dY ([kin][64]); dZ_{L-1} = (dY W_L) ⊙ SiLU'(Z_{L-1})
  Layer& o = s->L[nl - 1];
  int r = gemm(s, o.kin, kPadOut, B, s->Xt[nl - 1], s->dYt, EPI_F32, ACT_NONE, nullptr, o.gW, kPadOut, kPadOut, 0, nullptr, nullptr);
  if (r) return r;
  r = gemm(s, B, o.kin, kPadOut, s->dY, o.Wt, EPI_DACT, ACT_SILU, nullptr, s->dZ[nl - 1], o.kin, o.kin, 0, nullptr, s->Z[nl - 1],
           s->dZt[nl - 1], s->L[nl - 2].gb);
  if (r) return r;
  // hidden layers l = nl-2 .. 0: input X[l], output gradient dZ[l+1]
  for (int l = nl - 2; l >= 0; --l) {
    Layer& y = s->L[l];
    r = gemm(s, y.nrow, y.kin, B, s->dZt[l + 1], s->Xt[l], EPI_F32, ACT_NONE, nullptr, y.gW, y.kin, y.kin, 0, nullptr, nullptr);
    if (r) return r;
    if (l > 0) {
      r = gemm(s, B, y.kin, y.nrow, s->dZ[l + 1], y.Wt, EPI_DACT, ACT_SILU, nullptr, s->dZ[l], y.kin, y.kin, 0, nullptr, s->Z[l], s->dZt[l],
               s->L[l - 1].gb);
      if (r) return r;
    }
  }
  return cudaGetLastError() == cudaSuccess ? SBZ_OK : F(SBZ_ERR_CUDA, "surrogate: backward");
}

// forward + loss + backward of the `rows` rows in X[0] (and X[0]ᵀ) with targets T
int forward_backward(sbz_surrogate* s, int rows) {
  int r = forward(s, rows, true);
  if (r) return r;
  for (auto& l : s->L) SCU(cudaMemsetAsync(l.gb, 0, sizeof(float) * l.nrow, s->stream));
  loss_grad<<<(rows + kLossThreads - 1) / kLossThreads, kLossThreads, 0, s->stream>>>(rows, s->nout, s->Yf, s->L.back().b, s->T, s->dY, s->dYt,
                                                                                  s->L.back().gb, s->loss);
  return backward(s);
}

// one training step on the stream (captured into the step graph)
int train_step(sbz_surrogate* s) {
  const int B = s->batch;
  begin_step<<<1, 1, 0, s->stream>>>(s->dstep, s->loss);
  gather_batch<<<(B + 127) / 128, 128, 0, s->stream>>>(B, s->nin, s->nout, s->dataX, s->dataY, s->ndata, 0, s->dstep, s->seed, 0, 1, s->X[0],
                                                      s->Xt[0], s->T);
  int r = forward_backward(s, B);
  if (r) return r;
  adam_all<<<2 * 152, 256, 0, s->stream>>>(static_cast<const AdamSeg*>(s->segs), s->nseg, s->nparam_all, s->dstep, s->dlr, 0.9f, 0.999f,
                                           1e-8f);
  return cudaGetLastError() == cudaSuccess ? SBZ_OK : F(SBZ_ERR_CUDA, "surrogate: training step");
}

int check_err(sbz_surrogate* s) {
  unsigned e = 0;
  SCU(cudaMemcpyAsync(&e, s->err, sizeof e, cudaMemcpyDeviceToHost, s->stream));
  SCU(cudaStreamSynchronize(s->stream));
  return e ? F(SBZ_ERR_CUDA, "surrogate: GEMM pipeline wait ran out") : SBZ_OK;
}

// flat parameter order: per layer W [nout][nin] (logical, row-major) then b [nout]
long long nparams(const sbz_surrogate* s) {
  long long n = 0;
  for (auto& l : s->L) n += (long long)l.nout * l.nin + l.nout;
  return n;
}

}  // namespace

extern "C" {

int sbz_surrogate_create(int nin, int width, int nhidden, int nout, int batch, unsigned long long seed, sbz_surrogate** out) {
  if (!out || nin < 1 || nin > kPadIn || nout < 1 || nout > kPadOut || width < 128 || width % 128 || nhidden < 1 || batch < 128 ||
      batch % 128)
    return F(SBZ_ERR_ARG, "sbz_surrogate_create: need 1 <= nin, nout <= 64, width % 128 == 0, nhidden >= 1, batch % 128 == 0");
  auto* s = new sbz_surrogate();
  s->nin = nin; s->width = width; s->nhidden = nhidden; s->nout = nout; s->batch = batch; s->seed = seed;
  auto bail = [&](const char* m) { free_all(s); delete s; return F(SBZ_ERR_CUDA, m); };
  if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) return bail("surrogate: stream");
  const int nl = nhidden + 1;
  s->L.resize(nl);
  unsigned long long rs = seed * 0x2545F4914F6CDD1Dull + 1;
  for (int l = 0; l < nl; ++l) {
    Layer& y = s->L[l];
    y = Layer{};
    y.nin = l == 0 ? nin : width;
    y.kin = l == 0 ? kPadIn : width;
    y.nout = l == nl - 1 ? nout : width;
    y.nrow = l == nl - 1 ? kPadOut : width;
    y.gT = l == nl - 1;
    const size_t nw = (size_t)y.nrow * y.kin;
    if (dalloc(&y.W, nw) || dalloc(&y.mW, nw) || dalloc(&y.vW, nw) || dalloc(&y.gW, nw) || dalloc(&y.b, y.nrow) || dalloc(&y.mb, y.nrow) ||
        dalloc(&y.vb, y.nrow) || dalloc(&y.gb, y.nrow) || dalloc(&y.Wh, nw) || dalloc(&y.Wt, nw))
      return bail("surrogate: weight allocation");
    // Glorot-uniform weights on the logical block, zero padding and biases
    std::vector<float> w(nw, 0.0f);
    const float a = std::sqrt(6.0f / (float)(y.nin + y.nout));
    for (int r = 0; r < y.nout; ++r)
      for (int k = 0; k < y.nin; ++k) w[(size_t)r * y.kin + k] = a * (2.0f * (float)((splitmix(rs) >> 11) * 0x1.0p-53) - 1.0f);
    cudaMemcpy(y.W, w.data(), sizeof(float) * nw, cudaMemcpyHostToDevice);
    cudaMemset(y.b, 0, sizeof(float) * y.nrow);
    for (float* p : {y.mW, y.vW, y.gW}) cudaMemset(p, 0, sizeof(float) * nw);
    for (float* p : {y.mb, y.vb, y.gb}) cudaMemset(p, 0, sizeof(float) * y.nrow);
  }
  s->X.assign(nl, nullptr); s->Z.assign(nl, nullptr); s->Xt.assign(nl, nullptr); s->dZ.assign(nl, nullptr); s->dZt.assign(nl, nullptr);
  for (int l = 0; l < nl; ++l) {
    const int w = l == 0 ? kPadIn : width;
    if (dalloc(&s->X[l], (size_t)batch * w) || dalloc(&s->Xt[l], (size_t)batch * w)) return bail("surrogate: activation allocation");
    if (l > 0 && (dalloc(&s->Z[l], (size_t)batch * w) || dalloc(&s->dZ[l], (size_t)batch * w) || dalloc(&s->dZt[l], (size_t)batch * w)))
      return bail("surrogate: activation allocation");
  }
  if (dalloc(&s->Yf, (size_t)batch * kPadOut) || dalloc(&s->dY, (size_t)batch * kPadOut) || dalloc(&s->dYt, (size_t)batch * kPadOut) ||
      dalloc(&s->T, (size_t)batch * nout) || dalloc(&s->loss, 1) || dalloc(&s->err, 1))
    return bail("surrogate: buffer allocation");
  cudaMemset(s->err, 0, sizeof(unsigned));
  {
    std::vector<AdamSeg> segs;
    long long start = 0;
    for (auto& l : s->L) {
      const int n = l.nrow * l.kin;
      segs.push_back(AdamSeg{l.W, l.mW, l.vW, l.gW, l.Wh, l.Wt, start, n, l.gT ? 1 : 0, l.nrow, l.kin});
      start += n;
      segs.push_back(AdamSeg{l.b, l.mb, l.vb, l.gb, nullptr, nullptr, start, l.nrow, 0, l.nrow, 1});
      start += l.nrow;
    }
    s->nseg = (int)segs.size();
    s->nparam_all = start;
    if (dalloc(&s->dstep, 1) || dalloc(&s->dlr, 1) || cudaMalloc(&s->segs, sizeof(AdamSeg) * segs.size()) != cudaSuccess)
      return bail("surrogate: buffer allocation");
    cudaMemcpy(s->segs, segs.data(), sizeof(AdamSeg) * segs.size(), cudaMemcpyHostToDevice);
    cudaMemset(s->dstep, 0, sizeof(long long));
  }
  if (refresh_bf16(s) != SBZ_OK) { free_all(s); delete s; return SBZ_ERR_CUDA; }
  if (cudaStreamSynchronize(s->stream) != cudaSuccess) return bail("surrogate: initialisation");
  *out = s;
  return SBZ_OK;
}

void sbz_surrogate_destroy(sbz_surrogate* s) {
  if (!s) return;
  if (s->stream) cudaStreamSynchronize(s->stream);
  free_all(s);
  delete s;
}

long long sbz_surrogate_nparams(const sbz_surrogate* s) { return s ? nparams(s) : 0; }

int sbz_surrogate_get_params(const sbz_surrogate* s, float* params) {
  if (!s || !params) return F(SBZ_ERR_ARG, "null argument");
  long long o = 0;
  for (auto& l : s->L) {
    std::vector<float> w((size_t)l.nrow * l.kin), b(l.nrow);
    SCU(cudaMemcpy(w.data(), l.W, sizeof(float) * w.size(), cudaMemcpyDeviceToHost));
    SCU(cudaMemcpy(b.data(), l.b, sizeof(float) * b.size(), cudaMemcpyDeviceToHost));
    for (int r = 0; r < l.nout; ++r)
      for (int k = 0; k < l.nin; ++k) params[o++] = w[(size_t)r * l.kin + k];
    for (int r = 0; r < l.nout; ++r) params[o++] = b[r];
  }
  return SBZ_OK;
}

int sbz_surrogate_set_params(sbz_surrogate* s, const float* params) {
  if (!s || !params) return F(SBZ_ERR_ARG, "null argument");
  long long o = 0;
  for (auto& l : s->L) {
    std::vector<float> w((size_t)l.nrow * l.kin, 0.0f), b(l.nrow, 0.0f);
    for (int r = 0; r < l.nout; ++r)
      for (int k = 0; k < l.nin; ++k) w[(size_t)r * l.kin + k] = params[o++];
    for (int r = 0; r < l.nout; ++r) b[r] = params[o++];
    SCU(cudaMemcpy(l.W, w.data(), sizeof(float) * w.size(), cudaMemcpyHostToDevice));
    SCU(cudaMemcpy(l.b, b.data(), sizeof(float) * b.size(), cudaMemcpyHostToDevice));
  }
  int r = refresh_bf16(s);
  if (r) return r;
  SCU(cudaStreamSynchronize(s->stream));
  return SBZ_OK;
}

int sbz_surrogate_set_data(sbz_surrogate* s, long long n, const float* X, const float* Y) {
  if (!s || n < 1 || !X || !Y) return F(SBZ_ERR_ARG, "sbz_surrogate_set_data: bad arguments");
  if (s->stream) cudaStreamSynchronize(s->stream);
  if (s->graph_exec) { cudaGraphExecDestroy(s->graph_exec); s->graph_exec = nullptr; }
  if (s->graph) { cudaGraphDestroy(s->graph); s->graph = nullptr; }
  if (s->dataX) cudaFree(s->dataX);
  if (s->dataY) cudaFree(s->dataY);
  s->dataX = s->dataY = nullptr;
  SCU(dalloc(&s->dataX, (size_t)n * s->nin));
  SCU(dalloc(&s->dataY, (size_t)n * s->nout));
  SCU(cudaMemcpy(s->dataX, X, sizeof(float) * n * s->nin, cudaMemcpyHostToDevice));
  SCU(cudaMemcpy(s->dataY, Y, sizeof(float) * n * s->nout, cudaMemcpyHostToDevice));
  s->ndata = n;
  return SBZ_OK;
}

int sbz_surrogate_train(sbz_surrogate* s, int nsteps, double lr, double* loss_out) {
  if (!s || nsteps < 0 || !(lr > 0)) return F(SBZ_ERR_ARG, "sbz_surrogate_train: bad arguments");
  if (!s->dataX) return F(SBZ_ERR_STATE, "sbz_surrogate_train: no training data (sbz_surrogate_set_data)");
  set_value<<<1, 1, 0, s->stream>>>(s->dlr, (float)lr);
  int r = SBZ_OK;
  if (!s->graph_exec && nsteps > 0) {
    // the first step runs eagerly (kernel attributes, tensor-map encoder), the next is captured
    if ((r = train_step(s))) return r;
    ++s->step;
    --nsteps;
    SCU(cudaStreamSynchronize(s->stream));
    SCU(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    r = train_step(s);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(s->stream, &g);
    if (r || e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return r ? r : F(SBZ_ERR_CUDA, std::string("surrogate: step capture: ") + cudaGetErrorString(e));
    }
    s->graph = g;
    SCU(cudaGraphInstantiate(&s->graph_exec, s->graph, 0));
  }
  for (int it = 0; it < nsteps; ++it) SCU(cudaGraphLaunch(s->graph_exec, s->stream));
  s->step += nsteps;
  if (loss_out) SCU(cudaMemcpyAsync(loss_out, s->loss, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  return check_err(s);
}

int sbz_surrogate_gradients(sbz_surrogate* s, int n, const float* X, const float* Y, double* loss, float* grads) {
  if (!s || n < 1 || n > s->batch || n % 128 || !X || !Y) return F(SBZ_ERR_ARG, "sbz_surrogate_gradients: n % 128 == 0, n <= batch");
  // run one forward/backward on exactly these n rows (batch rows beyond n are zero inputs with zero
  // targets and do not contribute: their loss terms are excluded by using batch = n below)
  const int keepB = s->batch;
  s->batch = n;
  float *dx = nullptr, *dy = nullptr;
  SCU(dalloc(&dx, (size_t)n * s->nin));
  SCU(dalloc(&dy, (size_t)n * s->nout));
  SCU(cudaMemcpy(dx, X, sizeof(float) * n * s->nin, cudaMemcpyHostToDevice));
  SCU(cudaMemcpy(dy, Y, sizeof(float) * n * s->nout, cudaMemcpyHostToDevice));
  gather_batch<<<(n + 127) / 128, 128, 0, s->stream>>>(n, s->nin, s->nout, dx, dy, n, 0, nullptr, 0, 0, 0, s->X[0], s->Xt[0], s->T);
  cudaMemsetAsync(s->loss, 0, sizeof(double), s->stream);
  int r = forward_backward(s, n);
  s->batch = keepB;
  cudaFree(dx); cudaFree(dy);
  if (r) return r;
  if ((r = check_err(s))) return r;
  if (loss) SCU(cudaMemcpy(loss, s->loss, sizeof(double), cudaMemcpyDeviceToHost));
  if (grads) {
    long long o = 0;
    for (auto& l : s->L) {
      std::vector<float> g((size_t)l.nrow * l.kin), b(l.nrow);
      SCU(cudaMemcpy(g.data(), l.gW, sizeof(float) * g.size(), cudaMemcpyDeviceToHost));
      SCU(cudaMemcpy(b.data(), l.gb, sizeof(float) * b.size(), cudaMemcpyDeviceToHost));
      for (int rr = 0; rr < l.nout; ++rr)
        for (int k = 0; k < l.nin; ++k) grads[o++] = l.gT ? g[(size_t)k * l.nrow + rr] : g[(size_t)rr * l.kin + k];
      for (int rr = 0; rr < l.nout; ++rr) grads[o++] = b[rr];
    }
  }
  return SBZ_OK;
}

int sbz_surrogate_infer(sbz_surrogate* s, long long n, const float* X, float* Y) {
  if (!s || n < 0 || (n && (!X || !Y))) return F(SBZ_ERR_ARG, "sbz_surrogate_infer: bad arguments");
  if (n == 0) return SBZ_OK;
  const int B = s->batch;
  float *dx = nullptr, *dyo = nullptr;
  const long long chunk = std::min<long long>(n, 1ll << 22);
  SCU(dalloc(&dx, (size_t)chunk * s->nin));
  SCU(dalloc(&dyo, (size_t)B * s->nout));
  int r = SBZ_OK;
  for (long long c0 = 0; c0 < n && !r; c0 += chunk) {
    const long long cn = std::min(chunk, n - c0);
    if (cudaMemcpyAsync(dx, X + c0 * s->nin, sizeof(float) * cn * s->nin, cudaMemcpyHostToDevice, s->stream) != cudaSuccess) { r = SBZ_ERR_CUDA; break; }
    for (long long b0 = 0; b0 < cn && !r; b0 += B) {
      const int rows = (int)std::min<long long>(B, cn - b0);
      const int prow = (rows + 127) / 128 * 128;
      gather_batch<<<(prow + 127) / 128, 128, 0, s->stream>>>(prow, s->nin, s->nout, dx + b0 * s->nin, nullptr, rows, 0, nullptr, 0, 0, 0, s->X[0],
                                                              nullptr, nullptr);
      if ((r = forward(s, prow, false))) break;
      add_bias_out<<<(rows * s->nout + 255) / 256, 256, 0, s->stream>>>(rows, s->nout, s->Yf, s->L.back().b, dyo);
      if (cudaMemcpyAsync(Y + (c0 + b0) * s->nout, dyo, sizeof(float) * rows * s->nout, cudaMemcpyDeviceToHost, s->stream) != cudaSuccess)
        r = SBZ_ERR_CUDA;
    }
  }
  cudaStreamSynchronize(s->stream);
  cudaFree(dx); cudaFree(dyo);
  if (r) return r == SBZ_ERR_CUDA ? F(r, "sbz_surrogate_infer: copy") : r;
  return check_err(s);
}

// flat binary: "SBZMLP01", int32 nin, width, nhidden, nout, then the FP32 parameters in
// sbz_surrogate_get_params order (little-endian)
int sbz_surrogate_save(const sbz_surrogate* s, const char* path) {
  if (!s || !path) return F(SBZ_ERR_ARG, "null argument");
  std::vector<float> p((size_t)nparams(s));
  int r = sbz_surrogate_get_params(s, p.data());
  if (r) return r;
  FILE* f = std::fopen(path, "wb");
  if (!f) return F(SBZ_ERR_ARG, std::string("cannot write ") + path);
  const int hdr[4] = {s->nin, s->width, s->nhidden, s->nout};
  bool ok = std::fwrite("SBZMLP01", 1, 8, f) == 8 && std::fwrite(hdr, sizeof(int), 4, f) == 4 &&
            std::fwrite(p.data(), sizeof(float), p.size(), f) == p.size();
  ok = (std::fclose(f) == 0) && ok;
  return ok ? SBZ_OK : F(SBZ_ERR_ARG, std::string("write failed: ") + path);
}

int sbz_surrogate_load(const char* path, int batch, sbz_surrogate** out) {
  if (!path || !out) return F(SBZ_ERR_ARG, "null argument");
  FILE* f = std::fopen(path, "rb");
  if (!f) return F(SBZ_ERR_ARG, std::string("cannot read ") + path);
  char magic[8];
  int hdr[4];
  if (std::fread(magic, 1, 8, f) != 8 || std::memcmp(magic, "SBZMLP01", 8) || std::fread(hdr, sizeof(int), 4, f) != 4) {
    std::fclose(f);
    return F(SBZ_ERR_ARG, "not a surrogate weight file");
  }
  sbz_surrogate* s = nullptr;
  int r = sbz_surrogate_create(hdr[0], hdr[1], hdr[2], hdr[3], batch, 0, &s);
  if (r) { std::fclose(f); return r; }
  std::vector<float> p((size_t)nparams(s));
  const bool ok = std::fread(p.data(), sizeof(float), p.size(), f) == p.size();
  std::fclose(f);
  if (!ok) { sbz_surrogate_destroy(s); return F(SBZ_ERR_ARG, "truncated surrogate weight file"); }
  if ((r = sbz_surrogate_set_params(s, p.data()))) { sbz_surrogate_destroy(s); return r; }
  *out = s;
  return SBZ_OK;
}

}  // extern "C"
