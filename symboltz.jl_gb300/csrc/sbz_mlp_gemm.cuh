// BF16 tensor-core GEMM for the source surrogate's dense layers (sm_103a: TMA + tcgen05 + TMEM).
//
//   D[M x N] = A[M x K] · B[N x K]ᵀ   (A, B bf16 row-major with K contiguous, FP32 accumulation)
//
// One CTA computes a 128 x BN tile; two CTAs share an SM (≈ 100 KB of shared memory and at most
// 128 registers per thread each), so one CTA's epilogue overlaps the other's loads.  Warp 0 lane 0
// streams 128 x 64 and BN x 64 K-slices into a shared-memory ring of stages_for<BN>() slots with
// TMA (128-byte swizzle); warp 1 lane 0 issues
// tcgen05.mma (kind::f16, M = 128, N = BN, K = 16) into a TMEM accumulator and releases ring
// slots with tcgen05.commit; all eight warps then read the accumulator with tcgen05.ld (warp w owns
// TMEM lanes 32(w mod 4).. = tile rows, and half w / 4 of the tile's columns) and apply the fused
// epilogue:
//   EPI_F32   out_f32 = D (+ out_f32 when accumulate; split-K CTAs add with 16-byte atomics)
//   EPI_ACT   z = D + bias; out = bf16(act(z)); optional z_out = bf16(z)    forward layers
//   EPI_DACT  out = bf16(D · act'(z_in))                                   backward layers
// EPI_ACT / EPI_DACT can also store the output transposed (out_t[col][row], the operand layout of
// the weight-gradient GEMMs: a warp writes 32 consecutive rows of a column, pairs of rows packed
// into 4-byte stores) and, for EPI_DACT, add its column sums into colsum (the bias gradient).
// Every mbarrier wait is bounded: a wait that runs out sets *err and the CTA skips ahead to its
// TMEM release, so a fault in the pipeline cannot hang the GPU.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cstdint>

namespace sbz {
namespace mlp {

constexpr int BM = 128, BK = 64, kThreads = 256;
template <int BN>
__host__ __device__ constexpr int stages_for() { return BN >= 256 ? 2 : BN >= 128 ? 3 : 4; }  // (BM + BN) · BK · 2 B · stages ≤ 96 KB
constexpr unsigned kWaitLimit = 1u << 24;
enum { EPI_F32 = 0, EPI_ACT = 1, EPI_DACT = 2 };
enum { ACT_NONE = 0, ACT_SILU = 1 };

struct GemmArgs {
  int M, N, K;
  int epi, act;
  const float* bias;            // [N] (EPI_ACT), may be null
  __nv_bfloat16* out_bf16;      // EPI_ACT / EPI_DACT
  float* out_f32;               // EPI_F32
  int ldo;                      // output row stride (elements)
  int n_valid;                  // columns < n_valid are stored
  int accumulate;               // EPI_F32: add to the output
  __nv_bfloat16* z_out;         // EPI_ACT: pre-activation (ldo stride), may be null
  const __nv_bfloat16* z_in;    // EPI_DACT: pre-activation of this layer (ldo stride)
  __nv_bfloat16* out_t;         // EPI_ACT / EPI_DACT: transposed output, (col, row) at col * ldt + row; may be null
  int ldt;                      // its row stride (even)
  float* colsum;                // EPI_DACT: colsum[col] += Σ_rows out (as stored, bf16-rounded); may be null
  unsigned* err;                // set to 1 by a CTA whose pipeline wait ran out
};

template <int BN>
constexpr size_t gemm_smem_bytes() {
  constexpr int STAGES = stages_for<BN>();
  return 1024 /* alignment slack */ + (size_t)STAGES * (BM + BN) * BK * 2 + (2 * STAGES + 1) * 8 + 16 + BN * 4 /* bias */;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity) {
  const uint32_t a = smem_u32(b);
  for (unsigned i = 0; i < kWaitLimit; ++i) {
    uint32_t ready;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ready)
        : "r"(a), "r"(parity)
        : "memory");
    if (ready) return true;
  }
  return false;
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* tm, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// shared-memory matrix descriptor: K-major tile written by TMA with 128-byte swizzle
// (rows of 128 B, 8-row groups 1024 B apart), start address in 16-byte units
__device__ __forceinline__ uint64_t desc_sw128(const void* p) {
  uint64_t d = (uint64_t)((smem_u32(p) & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;            // leading-dimension offset (unused by swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;  // stride-dimension offset: next 8-row group
  d |= (uint64_t)1 << 46;            // descriptor version
  d |= (uint64_t)2 << 61;            // 128-byte swizzle
  return d;
}

template <int BN>
__device__ __forceinline__ uint32_t idesc_bf16() {
  return (1u << 4)                    // D: FP32
         | (1u << 7) | (1u << 10)     // A, B: BF16
         | ((uint32_t)(BN >> 3) << 17) // N
         | ((uint32_t)(BM >> 4) << 24); // M
}

// SiLU and its derivative with the fast exponential and division (the results are rounded to
// bf16; for z < -87 e^{-z} overflows to inf and both give the correct limit 0)
__device__ __forceinline__ float silu(float z) { return __fdividef(z, 1.0f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
  const float s = __fdividef(1.0f, 1.0f + __expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

// lane l ends with the sum over the warp's 32 lanes of a[l] (a transposing butterfly, 31 shuffles)
__device__ __forceinline__ float warp_column_sum(float (&a)[32], int lane) {
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) {
    const bool up = (lane & off) != 0;
#pragma unroll
    for (int i = 0; i < off; ++i) {
      const float send = up ? a[i] : a[i + off];
      const float keep = up ? a[i + off] : a[i];
      a[i] = keep + __shfl_xor_sync(0xffffffffu, send, off);
    }
  }
  return a[0];
}

__device__ __forceinline__ unsigned pack_bf16(float a, float b) {
  return (unsigned)__bfloat16_as_ushort(__float2bfloat16(a)) | ((unsigned)__bfloat16_as_ushort(__float2bfloat16(b)) << 16);
}
__device__ __forceinline__ float bf16_lo(unsigned u) { return __uint_as_float(u << 16); }
__device__ __forceinline__ float bf16_hi(unsigned u) { return __uint_as_float(u & 0xFFFF0000u); }

// transposed store of a warp's 32 rows x 32 columns (yp[p] = this lane's row, columns col0 + 2p and
// col0 + 2p + 1 packed): lanes 2i and 2i+1 swap halves so each stores two consecutive rows of one
// column as 4 bytes
__device__ __forceinline__ void store_transposed(const unsigned (&yp)[16], __nv_bfloat16* out_t, int ldt, int col0, int row, int ncol,
                                                 int lane) {
  const bool odd = lane & 1;
#pragma unroll
  for (int p = 0; p < 16; ++p) {
    const unsigned lo = yp[p] & 0xFFFFu, hi = yp[p] >> 16;
    const unsigned got = __shfl_xor_sync(0xffffffffu, odd ? lo : hi, 1);
    const int j = 2 * p + (odd ? 1 : 0);
    const unsigned pair = odd ? (got | (hi << 16)) : (lo | (got << 16));
    if (j < ncol) *reinterpret_cast<unsigned*>(out_t + (size_t)(col0 + j) * ldt + (row & ~1)) = pair;
  }
}

template <int BN>
__global__ void __launch_bounds__(kThreads, 2) gemm_tn_kernel(const __grid_constant__ CUtensorMap tmA,
                                                         const __grid_constant__ CUtensorMap tmB, GemmArgs g) {
  constexpr int STAGES = stages_for<BN>();
  extern __shared__ unsigned char smem_raw[];
  unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  unsigned char* sA = base;
  unsigned char* sB = sA + (size_t)STAGES * BM * BK * 2;
  uint64_t* full = (uint64_t*)(sB + (size_t)STAGES * BN * BK * 2);
  uint64_t* empty = full + STAGES;
  uint64_t* done = empty + STAGES;
  uint32_t* tmem_slot = (uint32_t*)(done + 1);
  float* sbias = (float*)(tmem_slot + 4);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n0 = blockIdx.x * BN, m0 = blockIdx.y * BM;
  // split-K (EPI_F32 only): CTA z owns K-steps [kt0, kt0 + KT) of the g.K / BK
  const int KTall = g.K / BK;
  const int kt0 = (int)((long long)KTall * blockIdx.z / gridDim.z);
  const int KT = (int)((long long)KTall * (blockIdx.z + 1) / gridDim.z) - kt0;
  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
    mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int j = threadIdx.x; j < BN; j += kThreads) sbias[j] = (g.bias && n0 + j < g.n_valid) ? g.bias[n0 + j] : 0.0f;
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)), "r"(BN) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  bool ok = true;
  if (warp == 0 && lane == 0) {  // TMA producer
    for (int kt = 0; kt < KT; ++kt) {
      const int s = kt % STAGES;
      const uint32_t ph = (uint32_t)(kt / STAGES) & 1u;
      if (!mbar_wait(&empty[s], ph ^ 1u)) { ok = false; break; }
      mbar_expect_tx(&full[s], (unsigned)((BM + BN) * BK * 2));
      tma_load_2d(sA + (size_t)s * BM * BK * 2, &tmA, (kt0 + kt) * BK, m0, &full[s]);
      tma_load_2d(sB + (size_t)s * BN * BK * 2, &tmB, (kt0 + kt) * BK, n0, &full[s]);
    }
  } else if (warp == 1 && lane == 0) {  // MMA issuer
    const uint32_t idesc = idesc_bf16<BN>();
    for (int kt = 0; kt < KT; ++kt) {
      const int s = kt % STAGES;
      const uint32_t ph = (uint32_t)(kt / STAGES) & 1u;
      if (!mbar_wait(&full[s], ph)) { ok = false; break; }
      tc_fence_after();
      const uint64_t ad = desc_sw128(sA + (size_t)s * BM * BK * 2), bd = desc_sw128(sB + (size_t)s * BN * BK * 2);
#pragma unroll
      for (int kk = 0; kk < BK / 16; ++kk) {  // advance 16 elements = 32 B inside the swizzled row
        const uint32_t acc = (kt | kk) != 0;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
            "l"(ad + 2 * kk), "l"(bd + 2 * kk), "r"(idesc), "r"(acc)
            : "memory");
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(&empty[s])) : "memory");
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(done)) : "memory");
  }
  __syncwarp();
  // epilogue: thread = tile row m0 + 32 (warp mod 4) + lane, columns of half warp / 4
  if (!mbar_wait(done, 0)) ok = false;
  ok = __syncthreads_and(ok) != 0;  // CTA-uniform: the TMEM loads below are warp-collective
  tc_fence_after();
  const int quarter = warp & 3, half = warp >> 2;
  const int row = m0 + quarter * 32 + lane;
  if (ok) {
#pragma unroll 1
    for (int c0 = half * (BN / 2); c0 < (half + 1) * (BN / 2); c0 += 32) {
      uint32_t v[32];
      const uint32_t taddr = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%"
          "22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]),
            "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]),
            "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]),
            "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      const int col = n0 + c0;
      if (col >= g.n_valid) continue;  // warp-uniform
      const bool live = row < g.M;
      const size_t o = (size_t)row * g.ldo + col;
      const int nv = min(32, g.n_valid - col);
      const bool vec = nv == 32 && (g.ldo % 8) == 0;
      if (g.epi == EPI_F32) {
        if (!live) continue;
        float* out = g.out_f32 + o;
        if (gridDim.z > 1) {
          if (vec) {
#pragma unroll
            for (int q = 0; q < 8; ++q)
              atomicAdd(reinterpret_cast<float4*>(out) + q, make_float4(__uint_as_float(v[4 * q]), __uint_as_float(v[4 * q + 1]),
                                                                         __uint_as_float(v[4 * q + 2]), __uint_as_float(v[4 * q + 3])));
          } else {
#pragma unroll
            for (int j = 0; j < 32; ++j) if (j < nv) atomicAdd(out + j, __uint_as_float(v[j]));
          }
        } else {
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            if (j >= nv) continue;
            const float d = __uint_as_float(v[j]);
            out[j] = g.accumulate ? out[j] + d : d;
          }
        }
        continue;
      }
      unsigned yp[16];  // bf16 pairs of the stored row
      if (g.epi == EPI_ACT) {
        unsigned zp[16];
#pragma unroll
        for (int p = 0; p < 16; ++p) {
          const float z0 = __uint_as_float(v[2 * p]) + sbias[c0 + 2 * p], z1 = __uint_as_float(v[2 * p + 1]) + sbias[c0 + 2 * p + 1];
          zp[p] = pack_bf16(z0, z1);
          yp[p] = g.act == ACT_SILU ? pack_bf16(silu(z0), silu(z1)) : zp[p];
        }
        if (live) {
          if (vec) {
            uint4* dst = reinterpret_cast<uint4*>(g.out_bf16 + o);
#pragma unroll
            for (int q = 0; q < 4; ++q) dst[q] = make_uint4(yp[4 * q], yp[4 * q + 1], yp[4 * q + 2], yp[4 * q + 3]);
            if (g.z_out) {
              uint4* dz = reinterpret_cast<uint4*>(g.z_out + o);
#pragma unroll
              for (int q = 0; q < 4; ++q) dz[q] = make_uint4(zp[4 * q], zp[4 * q + 1], zp[4 * q + 2], zp[4 * q + 3]);
            }
          } else {
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              if (j >= nv) continue;
              const unsigned short yj = (unsigned short)((j & 1) ? yp[j >> 1] >> 16 : yp[j >> 1] & 0xFFFFu);
              const unsigned short zj = (unsigned short)((j & 1) ? zp[j >> 1] >> 16 : zp[j >> 1] & 0xFFFFu);
              g.out_bf16[o + j] = __ushort_as_bfloat16(yj);
              if (g.z_out) g.z_out[o + j] = __ushort_as_bfloat16(zj);
            }
          }
        }
      } else {  // EPI_DACT
        unsigned zp[16];
        if (live && vec) {
          const uint4* src = reinterpret_cast<const uint4*>(g.z_in + o);
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const uint4 t = src[q];
            zp[4 * q] = t.x; zp[4 * q + 1] = t.y; zp[4 * q + 2] = t.z; zp[4 * q + 3] = t.w;
          }
        } else {
#pragma unroll
          for (int p = 0; p < 16; ++p) {
            const unsigned a = (live && 2 * p < nv) ? (unsigned)__bfloat16_as_ushort(g.z_in[o + 2 * p]) : 0u;
            const unsigned b = (live && 2 * p + 1 < nv) ? (unsigned)__bfloat16_as_ushort(g.z_in[o + 2 * p + 1]) : 0u;
            zp[p] = a | (b << 16);
          }
        }
#pragma unroll
        for (int p = 0; p < 16; ++p) {
          const float d0 = (live && 2 * p < nv) ? __uint_as_float(v[2 * p]) : 0.0f;
          const float d1 = (live && 2 * p + 1 < nv) ? __uint_as_float(v[2 * p + 1]) : 0.0f;
          yp[p] = g.act == ACT_SILU ? pack_bf16(d0 * dsilu(bf16_lo(zp[p])), d1 * dsilu(bf16_hi(zp[p]))) : pack_bf16(d0, d1);
        }
        if (live) {
          if (vec) {
            uint4* dst = reinterpret_cast<uint4*>(g.out_bf16 + o);
#pragma unroll
            for (int q = 0; q < 4; ++q) dst[q] = make_uint4(yp[4 * q], yp[4 * q + 1], yp[4 * q + 2], yp[4 * q + 3]);
          } else {
#pragma unroll
            for (int j = 0; j < 32; ++j)
              if (j < nv) g.out_bf16[o + j] = __ushort_as_bfloat16((unsigned short)((j & 1) ? yp[j >> 1] >> 16 : yp[j >> 1] & 0xFFFFu));
          }
        }
        if (g.colsum) {  // warp-collective; rows beyond M contribute zeros
          float a[32];
#pragma unroll
          for (int p = 0; p < 16; ++p) { a[2 * p] = bf16_lo(yp[p]); a[2 * p + 1] = bf16_hi(yp[p]); }
          const float cs = warp_column_sum(a, lane);
          if (lane < nv) atomicAdd(g.colsum + col + lane, cs);
        }
      }
      if (g.out_t && m0 + quarter * 32 < g.M) store_transposed(yp, g.out_t, g.ldt, col, row, nv, lane);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN) : "memory");
  if (!ok && lane == 0) atomicExch(g.err, 1u);
}

}  // namespace mlp
}  // namespace sbz
