// surrogate.cu — training and inference kernels of the thermal model
// (surrogate.h) on the tcgen05 tensor cores, and the frame generators of the
// FE-coupled path that use it or the synthetic field it learns.
//
// Kernels:
//   mlp_gemm_kernel<EPI>  one hidden layer's GEMM over a batch, D = A B^T with
//                         bf16 operands loaded by TMA (128-byte swizzle), FP32
//                         accumulators in TMEM, and a fused epilogue:
//                         bias + SiLU (forward; row and transposed copies for
//                         the weight gradients), bias + SiLU + FP32 head +
//                         loss gradients (last layer), SiLU' (backward), or a
//                         split-K partial (weight gradients).
//   mlp_infer_kernel      the whole network per 128-query tile, persistent:
//                         Fourier features written into shared memory, four
//                         MMA layers with their weights streamed by TMA while
//                         the previous epilogue runs, the head in FP32.
//   plus feature encoding, reductions, Adam, data generation and the frame
//   generators (multi-track field, model frames with fallback).
// Every wait (mbarrier) is bounded; a wait that runs out sets *error and the
// block returns after releasing its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/amca3d.h"
#include "surrogate.h"
#include "thermal_field.cuh"
#include "umma.cuh"

namespace amca {
namespace sur {

using bf16 = __nv_bfloat16;
constexpr unsigned long long kWaitNs = 1000000000ull;  // 1 s: every mbarrier wait
constexpr int kErrWait = 1;

enum { kEpiFwd = 0, kEpiHead = 1, kEpiBwd = 2, kEpiPartial = 3 };

// fast reciprocal (MUFU) on an argument kept below 2^126 (z >= -80)
__device__ __forceinline__ float sigmoid(float z) { return __fdividef(1.0f, 1.0f + __expf(-fmaxf(z, -80.0f))); }
__device__ __forceinline__ float silu(float z) { return z * sigmoid(z); }
__device__ __forceinline__ float silu_grad(float z) {
  const float s = sigmoid(z);
  return s * (1.0f + z * (1.0f - s));
}

// Phase j of one raw input: sv = sin(2 pi f_j), cv = cos(2 pi f_j),
// f_j = sum_i B[j][i] u_i (FP32, i ascending), u = (raw - shift) * scale.
__device__ __forceinline__ void phases(const SurModelDev &m, const float raw[kSurIn], int j, float &sv, float &cv) {
  float u[kSurIn];
#pragma unroll
  for (int i = 0; i < kSurIn; ++i) u[i] = (raw[i] - m.in_shift[i]) * m.in_scale[i];
  float f = 0.0f;
#pragma unroll
  for (int i = 0; i < kSurIn; ++i) f = __fadd_rn(f, __fmul_rn(m.fourier[j * kSurIn + i], u[i]));
  sincospif(2.0f * f, &sv, &cv);
}

// ---------------------------------------------------------------------------
// Layer GEMM with fused epilogues (training). D[M x N] = A[M x K] * B[N x K]^T.
// Block: 256 threads; thread 0 issues the TMA loads and the MMAs; afterwards
// warp w reads TMEM lanes 32 (w % 4) .. +31 (rows) and columns of half w / 4.
// ---------------------------------------------------------------------------
constexpr int kStages = 4;

struct GemmArgs {
  int M, N, K;
  int kb_per_split;        // 64-wide K blocks per block (split-K over gridDim.z)
  const float *bias;       // [N]
  bf16 *out_row;           // [M x N]  H (forward) or dZ (backward)
  bf16 *out_t;             // [N x M]  transposed copy
  bf16 *head_t;            // [N x M]  last layer: its activations, transposed (head weight gradients)
  bf16 *z_row;             // [M x N]  pre-activation (forward)
  const bf16 *z_in;        // [M x N]  pre-activation of this output (backward)
  float *partial;          // [splits x M x N] (split-K)
  // last layer
  const float *Wh, *bh;    // head (2 x N, 2)
  const float *target;     // [M] normalised temperature
  float *pred;             // [M x 2] mu, s
  float *dpred;            // [M x 2] dL/dmu, dL/ds
  float *loss;             // [M]
  float inv_batch, lambda_s;
  int *error;
};

__device__ __forceinline__ uint8_t *align1024(uint8_t *p) {
  return (uint8_t *)(((uintptr_t)p + 1023) & ~(uintptr_t)1023);
}

template <int EPI>
__global__ void __launch_bounds__(256, 1)
    mlp_gemm_kernel(const __grid_constant__ CUtensorMap tA, const __grid_constant__ CUtensorMap tB, GemmArgs a) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = align1024(smem_raw);
  __shared__ __align__(8) uint64_t full[kStages], empty[kStages], done;
  __shared__ uint32_t tmem_base;
  __shared__ int s_abort;
  __shared__ float s_head[2][128][2];

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int N = a.N;
  const uint32_t a_bytes = 128u * 128u, b_bytes = (uint32_t)N * 128u, stage_bytes = a_bytes + b_bytes;
  const int m0 = blockIdx.x * 128;
  const int kb0 = blockIdx.z * a.kb_per_split, nk = a.kb_per_split;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      umma::mbar_init(umma::smem_u32(&full[s]), 1);
      umma::mbar_init(umma::smem_u32(&empty[s]), 1);
    }
    umma::mbar_init(umma::smem_u32(&done), 1);
    umma::mbar_fence_init();
    s_abort = 0;
  }
  if (warp == 0) umma::tmem_alloc(umma::smem_u32(&tmem_base), 256);
  umma::tc_fence_before();
  __syncthreads();
  umma::tc_fence_after();
  const uint32_t tmem = tmem_base;

  if (threadIdx.x == 0) {
    umma::tma_prefetch_desc(&tA);
    umma::tma_prefetch_desc(&tB);
    const uint32_t idesc = umma::idesc_bf16_f32(128, N);
    auto load = [&](int s, int kb) {
      const uint32_t sa = umma::smem_u32(smem + (size_t)s * stage_bytes), bar = umma::smem_u32(&full[s]);
      umma::mbar_expect_tx(bar, stage_bytes);
      umma::tma_load_2d(sa, &tA, bar, (kb0 + kb) * 64, m0);
      umma::tma_load_2d(sa + a_bytes, &tB, bar, (kb0 + kb) * 64, 0);
    };
    int loaded = 0;
    for (int s = 0; s < kStages && s < nk; ++s, ++loaded) load(s, s);
    bool ok = true;
    for (int kb = 0; kb < nk && ok; ++kb) {
      const int s = kb % kStages;
      if (!umma::mbar_wait(umma::smem_u32(&full[s]), (uint32_t)((kb / kStages) & 1), kWaitNs)) {
        ok = false;
        break;
      }
      umma::tc_fence_after();
      const uint32_t sa = umma::smem_u32(smem + (size_t)s * stage_bytes), sb = sa + a_bytes;
#pragma unroll
      for (int k = 0; k < 4; ++k)
        umma::mma_bf16(tmem, umma::sdesc_sw128(sa + 32u * k), umma::sdesc_sw128(sb + 32u * k), idesc,
                       (kb | k) != 0 ? 1u : 0u);
      umma::mma_commit(umma::smem_u32(&empty[s]));
      // refill the stage of the previous K block (its MMAs were issued one iteration earlier)
      const int kr = kb - 1 + kStages;
      if (kb >= 1 && kr < nk) {
        const int sp = (kb - 1) % kStages;
        if (!umma::mbar_wait(umma::smem_u32(&empty[sp]), (uint32_t)(((kb - 1) / kStages) & 1), kWaitNs)) {
          ok = false;
          break;
        }
        load(sp, kr);
        ++loaded;
      }
    }
    if (!ok) {
      s_abort = 1;
      atomicCAS(a.error, 0, kErrWait);
      // let every load still in flight land before the block exits
      for (int kb = 0; kb < loaded; ++kb)
        umma::mbar_wait(umma::smem_u32(&full[kb % kStages]), (uint32_t)((kb / kStages) & 1), kWaitNs);
    }
    umma::mma_commit(umma::smem_u32(&done));  // arrives once every MMA issued above has completed
  }
  const bool done_ok = umma::mbar_wait(umma::smem_u32(&done), 0, kWaitNs);
  const bool all_ok = __syncthreads_and(done_ok ? 1 : 0) != 0;
  if (!done_ok) atomicCAS(a.error, 0, kErrWait);
  umma::tc_fence_after();

  if (all_ok && !s_abort) {
    const int q = warp & 3, half = warp >> 2;
    const int row = q * 32 + lane, m = m0 + row;
    const uint32_t trow = tmem + ((uint32_t)(q * 32) << 16);
    const int cols = N / 2, cbeg = half * cols;
    if (EPI == kEpiPartial) {
      float *dst = a.partial + ((size_t)blockIdx.z * a.M + m) * N;
      for (int c0 = cbeg; c0 < cbeg + cols; c0 += 32) {
        float v[32];
        umma::tmem_ld32(trow + c0, v);
#pragma unroll
        for (int j = 0; j < 32; j += 4) *(float4 *)(dst + c0 + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
      }
    } else if (EPI == kEpiFwd) {
      for (int c0 = cbeg; c0 < cbeg + cols; c0 += 32) {
        float v[32];
        umma::tmem_ld32(trow + c0, v);
        __align__(16) bf16 zb[32], hb[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const float z = v[j] + a.bias[c0 + j];
          const float h = silu(z);
          zb[j] = __float2bfloat16_rn(z);
          hb[j] = __float2bfloat16_rn(h);
          a.out_t[(size_t)(c0 + j) * a.M + m] = hb[j];
        }
#pragma unroll
        for (int j = 0; j < 32; j += 8) {
          *(uint4 *)(a.z_row + (size_t)m * N + c0 + j) = *(const uint4 *)&zb[j];
          *(uint4 *)(a.out_row + (size_t)m * N + c0 + j) = *(const uint4 *)&hb[j];
        }
      }
    } else if (EPI == kEpiBwd) {
      for (int c0 = cbeg; c0 < cbeg + cols; c0 += 32) {
        float v[32];
        umma::tmem_ld32(trow + c0, v);
        __align__(16) bf16 zb[32], gb[32];
#pragma unroll
        for (int j = 0; j < 32; j += 8) *(uint4 *)&zb[j] = *(const uint4 *)(a.z_in + (size_t)m * N + c0 + j);
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          gb[j] = __float2bfloat16_rn(v[j] * silu_grad(__bfloat162float(zb[j])));
          a.out_t[(size_t)(c0 + j) * a.M + m] = gb[j];
        }
        if (a.out_row) {
#pragma unroll
          for (int j = 0; j < 32; j += 8) *(uint4 *)(a.out_row + (size_t)m * N + c0 + j) = *(const uint4 *)&gb[j];
        }
      }
    } else {  // kEpiHead: last hidden layer, FP32 head, loss gradients, then dZ of this layer
      float mu = 0.0f, s = 0.0f;
      for (int c0 = cbeg; c0 < cbeg + cols; c0 += 32) {
        float v[32];
        umma::tmem_ld32(trow + c0, v);
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const float h = silu(v[j] + a.bias[c0 + j]);
          a.head_t[(size_t)(c0 + j) * a.M + m] = __float2bfloat16_rn(h);
          mu = fmaf(h, a.Wh[c0 + j], mu);
          s = fmaf(h, a.Wh[N + c0 + j], s);
        }
      }
      s_head[half][row][0] = mu;
      s_head[half][row][1] = s;
      __syncthreads();
      mu = s_head[0][row][0] + s_head[1][row][0] + a.bh[0];
      s = s_head[0][row][1] + s_head[1][row][1] + a.bh[1];
      s = fminf(fmaxf(s, -12.0f), 4.0f);
      const float y = a.target[m];
      const float r = mu - y;
      const float e2 = __expf(-2.0f * s);
      // mean squared error on mu; the error head learns log |mu - y| (Gaussian
      // negative log-likelihood with mu held fixed), weighted by lambda_s
      const float dmu = r * a.inv_batch;
      const float ds = a.lambda_s * (1.0f - e2 * r * r) * a.inv_batch;
      if (half == 0) {
        a.pred[2 * (size_t)m] = mu;
        a.pred[2 * (size_t)m + 1] = s;
        a.dpred[2 * (size_t)m] = dmu;
        a.dpred[2 * (size_t)m + 1] = ds;
        a.loss[m] = 0.5f * r * r;
      }
      for (int c0 = cbeg; c0 < cbeg + cols; c0 += 32) {
        float v[32];
        umma::tmem_ld32(trow + c0, v);
        __align__(16) bf16 gb[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const float dh = dmu * a.Wh[c0 + j] + ds * a.Wh[N + c0 + j];
          gb[j] = __float2bfloat16_rn(dh * silu_grad(v[j] + a.bias[c0 + j]));
          a.out_t[(size_t)(c0 + j) * a.M + m] = gb[j];
        }
#pragma unroll
        for (int j = 0; j < 32; j += 8) *(uint4 *)(a.out_row + (size_t)m * N + c0 + j) = *(const uint4 *)&gb[j];
      }
    }
  }
  umma::tc_fence_before();
  __syncthreads();
  if (warp == 0) umma::tmem_free(tmem, 256);
}

}  // namespace sur
}  // namespace amca

namespace amca {
namespace sur {

// ---------------------------------------------------------------------------
// Training helpers
// ---------------------------------------------------------------------------

// E[m][0..127] and its transpose from raw inputs (rows past n are zero).
__global__ void encode_kernel(SurModelDev md, const float *raw, int64_t n, int64_t M, bf16 *E, bf16 *Et) {
  const int64_t total = M * kSurFreq;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t m = q / kSurFreq;
    const int j = (int)(q % kSurFreq);
    float sv = 0.0f, cv = 0.0f;
    if (m < n) {
      float r[kSurIn];
#pragma unroll
      for (int i = 0; i < kSurIn; ++i) r[i] = raw[m * kSurIn + i];
      phases(md, r, j, sv, cv);
    }
    const bf16 s = __float2bfloat16_rn(sv), c = __float2bfloat16_rn(cv);
    E[m * kSurEnc + j] = s;
    E[m * kSurEnc + kSurFreq + j] = c;
    Et[(int64_t)j * M + m] = s;
    Et[(int64_t)(kSurFreq + j) * M + m] = c;
  }
}

// out[r] = sum over the `splits` partials of element r; a deterministic
// split-K reduction.
__global__ void reduce_partials_kernel(const float *partial, int splits, int64_t count, float *out) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < count; r += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.0f;
    for (int z = 0; z < splits; ++z) s += partial[(int64_t)z * count + r];
    out[r] = s;
  }
}

// out[r] = sum_m X[r][m] for a [rows x M] bf16 matrix (bias gradients from the
// transposed dZ); one block per row, fixed reduction order.
__global__ void row_sum_kernel(const bf16 *X, int64_t M, float *out) {
  __shared__ float red[256];
  const bf16 *x = X + (int64_t)blockIdx.x * M;
  float s = 0.0f;
  for (int64_t m = threadIdx.x; m < M; m += blockDim.x) s += __bfloat162float(x[m]);
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}

// Head gradients: gWh[j][c] = sum_m dpred[m][j] H[c][m], gbh[j] = sum_m dpred[m][j];
// one block per column c (plus one block for the biases).
__global__ void head_grad_kernel(const bf16 *Ht, const float *dpred, int64_t M, int N, float *gWh, float *gbh) {
  __shared__ float red[2][256];
  const int c = blockIdx.x;
  float s0 = 0.0f, s1 = 0.0f;
  for (int64_t m = threadIdx.x; m < M; m += blockDim.x) {
    const float h = c < N ? __bfloat162float(Ht[(int64_t)c * M + m]) : 1.0f;
    s0 += dpred[2 * m] * h;
    s1 += dpred[2 * m + 1] * h;
  }
  red[0][threadIdx.x] = s0;
  red[1][threadIdx.x] = s1;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      red[0][threadIdx.x] += red[0][threadIdx.x + w];
      red[1][threadIdx.x] += red[1][threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    if (c < N) {
      gWh[c] = red[0][0];
      gWh[N + c] = red[1][0];
    } else {
      gbh[0] = red[0][0];
      gbh[1] = red[1][0];
    }
  }
}

// Adam step over every parameter; refreshes the bf16 copies ([out][in] and,
// for layers 1.., the transposed [in][out] copy the backward GEMMs read).
struct AdamArgs {
  float *p, *m, *v;
  const float *g;
  int64_t n;
  float lr, beta1, beta2, eps, bc1, bc2;
  bf16 *Wb[kSurLayers], *Wtb[kSurLayers];
  int64_t Woff[kSurLayers];
};

__device__ __forceinline__ void store_bf16_copies(const AdamArgs &a, int64_t i, float p) {
#pragma unroll
  for (int l = 0; l < kSurLayers; ++l) {
    const int K = SurParamLayout::in_dim(l);
    const int64_t o = i - a.Woff[l];
    if (o >= 0 && o < (int64_t)kSurHid * K) {
      a.Wb[l][o] = __float2bfloat16_rn(p);
      if (a.Wtb[l]) a.Wtb[l][(o % K) * kSurHid + o / K] = __float2bfloat16_rn(p);
    }
  }
}

__global__ void adam_kernel(AdamArgs a) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.n; i += (int64_t)gridDim.x * blockDim.x) {
    const float g = a.g[i];
    const float m = a.beta1 * a.m[i] + (1.0f - a.beta1) * g;
    const float v = a.beta2 * a.v[i] + (1.0f - a.beta2) * g * g;
    a.m[i] = m;
    a.v[i] = v;
    const float p = a.p[i] - a.lr * (m / a.bc1) / (sqrtf(v / a.bc2) + a.eps);
    a.p[i] = p;
    store_bf16_copies(a, i, p);
  }
}

// bf16 copies of every layer's weights from the master parameters.
__global__ void refresh_bf16_kernel(AdamArgs a) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.n; i += (int64_t)gridDim.x * blockDim.x)
    store_bf16_copies(a, i, a.p[i]);
}

// acc[0] += sum of loss[0..n)
__global__ void accum_loss_kernel(const float *loss, int64_t n, double *acc) {
  __shared__ double red[256];
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s += loss[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(acc, red[0]);
}

// Counter-based uniform draws: (seed, stream, index) -> [0, 1), splitmix64.
__host__ __device__ inline uint64_t mix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
__host__ __device__ inline double uniform01(uint64_t seed, uint64_t stream, uint64_t i) {
  return (double)(mix64(seed * 0x100000001b3ull ^ mix64(stream * 0x9e3779b97f4a7c15ull + i)) >> 11) * 0x1.0p-53;
}

// Training set: sample i is a point at a random offset from the source (the
// frames of a moving source present FE nodes at every offset), at a random
// power and speed, labelled with the FE field. A fraction `near` of the
// samples is drawn from the box around the melt pool, a fraction `shell` from
// that box until the field lies in [shell_lo, shell_hi] (the band around the
// mushy zone), the rest from the model's window.
struct DataSpec {
  uint64_t seed;
  double p_lo, p_hi, v_lo, v_hi;
  double win_lo[3], win_hi[3];    // along-track, lateral, depth window (m)
  double near_lo[3], near_hi[3];  // melt-pool box (m)
  double near;                    // fraction from the melt-pool box
  double shell_lo, shell_hi;      // temperature band (K) ...
  double shell;                   // ... fraction of the samples drawn from the box until inside it
  ScanSource src;                 // physics; power and speed are replaced per sample
  float t_shift, t_scale;
  int log_out;
};

__global__ void make_data_kernel(DataSpec ds, int64_t first, int64_t n, float *raw, float *target) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t i = (uint64_t)(first + q);
    ScanSource s = ds.src;
    s.ntracks = 1;
    s.power = ds.p_lo + (ds.p_hi - ds.p_lo) * uniform01(ds.seed, 0, i);
    s.speed = ds.v_lo + (ds.v_hi - ds.v_lo) * uniform01(ds.seed, 1, i);
    const double kind = uniform01(ds.seed, 2, i);
    const bool shell = kind < ds.shell, nr = shell || kind < ds.shell + ds.near;
    // source at x = 0, y = 0 on the surface z = z_top = 0 at t = 0
    s.x_start = 0.0;
    s.y_line = 0.0;
    s.z_top = 0.0;
    double off[3] = {0.0, 0.0, 0.0}, T = 0.0;
    for (int attempt = 0; attempt < (shell ? 64 : 1); ++attempt) {
      for (int a = 0; a < 3; ++a) {
        const double lo = nr ? ds.near_lo[a] : ds.win_lo[a], hi = nr ? ds.near_hi[a] : ds.win_hi[a];
        off[a] = lo + (hi - lo) * uniform01(ds.seed, 3 + a + 8 * (uint64_t)attempt, i);
      }
      T = scan_field(s, off[0], off[1], -off[2], 0.0);
      if (T >= ds.shell_lo && T <= ds.shell_hi) break;
    }
    raw[q * kSurIn + 0] = (float)off[0];
    raw[q * kSurIn + 1] = (float)off[1];
    raw[q * kSurIn + 2] = (float)off[2];
    raw[q * kSurIn + 3] = (float)s.power;
    raw[q * kSurIn + 4] = (float)s.speed;
    const double yv = (T - ds.t_shift) / ds.t_scale;
    target[q] = (float)(ds.log_out ? log(yv) : yv);
  }
}

// Batch rows from the data set through an affine permutation:
// row q = data[(start + q) * perm_a mod n], perm_a coprime to n.
__global__ void gather_batch_kernel(const float *raw, const float *target, int64_t nsamples, int64_t start, int64_t nb,
                                    uint64_t perm_a, float *braw, float *btarget) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nb; q += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t i = (uint64_t)(((unsigned __int128)(uint64_t)(start + q) * perm_a) % (uint64_t)nsamples);
#pragma unroll
    for (int k = 0; k < kSurIn; ++k) braw[q * kSurIn + k] = raw[i * kSurIn + k];
    btarget[q] = target[i];
  }
}

// ---------------------------------------------------------------------------
// Frames on the FE node grid: the synthetic field of a scan, and the model.
// Node file coordinates are origin + spacing * index, the field is evaluated
// at file coordinate * length_scale, frame f at field time (f * frame_dt) *
// time_scale (the conventions of amca_set_rosenthal_frames).
// ---------------------------------------------------------------------------
struct FrameJob {
  ScanSource src;
  double origin[3], spacing;
  int nodes[3];
  double length_scale, frame_dt, time_scale;
  int f0, nf;                    // frames f0 .. f0 + nf - 1
  double *ring;                  // frame f goes to slot f % slots
  int slots;
  int64_t nnodes;
  // model frames only
  int box[3];                    // window size in nodes
  double win_lo[3], win_hi[3];   // window around the source (m): along-track, lateral, depth
  float t_liq, band, thresh;     // fallback: |T - t_liq| < band and error estimate > thresh (K)
  unsigned long long *counters;  // [0] nodes evaluated, [1] near the liquidus, [2] fallbacks
};

__device__ __forceinline__ void node_xyz(const FrameJob &j, int64_t n, double &x, double &y, double &z) {
  const int64_t I = n % j.nodes[0], J = (n / j.nodes[0]) % j.nodes[1], K = n / ((int64_t)j.nodes[0] * j.nodes[1]);
  x = (j.origin[0] + j.spacing * (double)I) * j.length_scale;
  y = (j.origin[1] + j.spacing * (double)J) * j.length_scale;
  z = (j.origin[2] + j.spacing * (double)K) * j.length_scale;
}

__device__ __forceinline__ double frame_time(const FrameJob &j, int f) { return ((double)f * j.frame_dt) * j.time_scale; }

// the synthetic field of the scan at every node of the frames
__global__ void scan_frames_kernel(FrameJob j) {
  const int64_t total = j.nnodes * j.nf;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int f = j.f0 + (int)(q / j.nnodes);
    const int64_t n = q % j.nnodes;
    double x, y, z;
    node_xyz(j, n, x, y, z);
    j.ring[(int64_t)(f % j.slots) * j.nnodes + n] = scan_field(j.src, x, y, z, frame_time(j, f));
  }
}

// every node of the frames at the ambient temperature (the model's value
// outside its window)
__global__ void fill_frames_kernel(FrameJob j) {
  const int64_t total = j.nnodes * j.nf;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int f = j.f0 + (int)(q / j.nnodes);
    j.ring[(int64_t)(f % j.slots) * j.nnodes + q % j.nnodes] = j.src.t0;
  }
}

// Query q of a model-frame job: its node (or -1 outside the grid) and frame.
__device__ __forceinline__ int64_t frame_query(const FrameJob &j, int64_t q, int &f) {
  const int64_t boxn = (int64_t)j.box[0] * j.box[1] * j.box[2];
  f = j.f0 + (int)(q / boxn);
  const int64_t l = q % boxn;
  const int bi = (int)(l % j.box[0]), bj = (int)((l / j.box[0]) % j.box[1]),
            bk = (int)(l / ((int64_t)j.box[0] * j.box[1]));
  double xl, yl, dir;
  scan_position(j.src, frame_time(j, f), xl, yl, dir);
  const double xmin = dir > 0 ? xl + j.win_lo[0] : xl - j.win_hi[0];
  const double ymin = yl + j.win_lo[1];
  const double zmin = j.src.z_top - j.win_hi[2];
  const int i0 = (int)floor((xmin / j.length_scale - j.origin[0]) / j.spacing);
  const int j0 = (int)floor((ymin / j.length_scale - j.origin[1]) / j.spacing);
  const int k0 = (int)floor((zmin / j.length_scale - j.origin[2]) / j.spacing);
  const int I = i0 + bi, J = j0 + bj, K = k0 + bk;
  if (I < 0 || I >= j.nodes[0] || J < 0 || J >= j.nodes[1] || K < 0 || K >= j.nodes[2]) return -1;
  return ((int64_t)K * j.nodes[1] + J) * j.nodes[0] + I;
}

// ---------------------------------------------------------------------------
// Fused inference: the whole network on 128-query tiles, persistent.
// Shared memory: activations H (128 x 256 bf16, four 64-column blocks of
// 16 KB) and one layer's weights (256 x 256 bf16, four blocks of 32 KB).
// 512 threads: warp w reads TMEM lanes 32 (w % 4) (its rows) and handles the
// 64-column group w / 4 of every layer's epilogue.
// ---------------------------------------------------------------------------
constexpr int kInferThreads = 512, kInferGroups = 4, kGroupCols = kSurHid / kInferGroups;
enum { kSrcArray = 0, kSrcFrames = 1 };

struct InferArgs {
  int64_t nq;
  const float *raw;  // kSrcArray: nq x 5 raw inputs
  float *T, *err;    // kSrcArray: outputs (K)
  FrameJob job;      // kSrcFrames
  int *error;
};

constexpr uint32_t kInferSmem = 64u * 1024u + 128u * 1024u + 1024u;

template <int SRC>
__global__ void __launch_bounds__(kInferThreads, 1)
    mlp_infer_kernel(const __grid_constant__ CUtensorMap tW0, const __grid_constant__ CUtensorMap tW1,
                     const __grid_constant__ CUtensorMap tW2, const __grid_constant__ CUtensorMap tW3, SurModelDev md,
                     InferArgs a) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t *H = align1024(smem_raw);
  uint8_t *Wsm = H + 64 * 1024;
  __shared__ __align__(8) uint64_t wbar, mbar;
  __shared__ uint32_t tmem_base;
  __shared__ int s_abort;
  __shared__ __align__(16) float s_bias[kSurLayers][kSurHid];
  __shared__ __align__(16) float s_wh[kSurOut][kSurHid];
  __shared__ float s_bh[kSurOut];
  __shared__ float s_head[kInferGroups][128][2];
  const CUtensorMap *tW[4] = {&tW0, &tW1, &tW2, &tW3};

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int q4 = warp & 3, grp = warp >> 2, row = q4 * 32 + lane;
  const int64_t ntiles = (a.nq + 127) / 128;
  const SurParamLayout L;

  for (int i = threadIdx.x; i < kSurLayers * kSurHid; i += blockDim.x)
    s_bias[i / kSurHid][i % kSurHid] = md.p[L.b[i / kSurHid] + i % kSurHid];
  for (int i = threadIdx.x; i < kSurOut * kSurHid; i += blockDim.x) s_wh[i / kSurHid][i % kSurHid] = md.p[L.Wh + i];
  if (threadIdx.x < kSurOut) s_bh[threadIdx.x] = md.p[L.bh + threadIdx.x];
  if (threadIdx.x == 0) {
    umma::mbar_init(umma::smem_u32(&wbar), 1);
    umma::mbar_init(umma::smem_u32(&mbar), 1);
    umma::mbar_fence_init();
    s_abort = 0;
  }
  if (warp == 0) umma::tmem_alloc(umma::smem_u32(&tmem_base), 256);
  umma::tc_fence_before();
  __syncthreads();
  umma::tc_fence_after();
  const uint32_t tmem = tmem_base;
  const uint32_t trow = tmem + ((uint32_t)(q4 * 32) << 16);
  const uint32_t idesc = umma::idesc_bf16_f32(128, kSurHid);

  auto load_w = [&](int l) {  // thread 0
    const int kbs = SurParamLayout::in_dim(l) / 64;
    const uint32_t bar = umma::smem_u32(&wbar);
    umma::mbar_expect_tx(bar, (uint32_t)kbs * 32u * 1024u);
    for (int kb = 0; kb < kbs; ++kb) umma::tma_load_2d(umma::smem_u32(Wsm + kb * 32 * 1024), tW[l], bar, kb * 64, 0);
  };
  if (threadIdx.x == 0) {
    for (int l = 0; l < 4; ++l) umma::tma_prefetch_desc(tW[l]);
    if ((int64_t)blockIdx.x < ntiles) load_w(0);
  }
  uint32_t wph = 0, mph = 0;
  bool ok = true;

  for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
    const int64_t qi = tile * 128 + row;
    bool valid = qi < a.nq;
    float raw[kSurIn] = {0, 0, 0, 0, 0};
    int f = 0;
    int64_t node = -1;
    double nx = 0, ny = 0, nz = 0;
    if (SRC == kSrcArray) {
      if (valid)
#pragma unroll
        for (int i = 0; i < kSurIn; ++i) raw[i] = a.raw[qi * kSurIn + i];
    } else if (valid) {
      node = frame_query(a.job, qi, f);
      valid = node >= 0;
      if (valid) {
        node_xyz(a.job, node, nx, ny, nz);
        scan_inputs(a.job.src, nx, ny, nz, frame_time(a.job, f), raw);
      }
    }
    // Fourier features: this group's 16 phases, sines at column j, cosines at 64 + j
    for (int j0 = grp * (kSurFreq / kInferGroups); j0 < (grp + 1) * (kSurFreq / kInferGroups); j0 += 8) {
      __align__(16) bf16 sb[8], cb[8];
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        float sv, cv;
        phases(md, raw, j0 + t, sv, cv);
        sb[t] = __float2bfloat16_rn(sv);
        cb[t] = __float2bfloat16_rn(cv);
      }
      *(uint4 *)(H + umma::sw128_offset(row, j0, 128)) = *(const uint4 *)sb;
      *(uint4 *)(H + umma::sw128_offset(row, kSurFreq + j0, 128)) = *(const uint4 *)cb;
    }
    umma::fence_async_smem();
    umma::tc_fence_before();
    __syncthreads();
    float mu = 0.0f, sl = 0.0f;
    for (int l = 0; l < kSurLayers; ++l) {
      if (threadIdx.x == 0) {
        const bool wok = umma::mbar_wait(umma::smem_u32(&wbar), wph, kWaitNs);
        if (!wok) {
          s_abort = 1;
        } else {
          umma::tc_fence_after();
          const int kbs = SurParamLayout::in_dim(l) / 64;
          for (int kb = 0; kb < kbs; ++kb) {
            const uint32_t ha = umma::smem_u32(H + kb * 16 * 1024), wa = umma::smem_u32(Wsm + kb * 32 * 1024);
#pragma unroll
            for (int k = 0; k < 4; ++k)
              umma::mma_bf16(tmem, umma::sdesc_sw128(ha + 32u * k), umma::sdesc_sw128(wa + 32u * k), idesc,
                             (kb | k) != 0 ? 1u : 0u);
          }
        }
        umma::mma_commit(umma::smem_u32(&mbar));
      }
      wph ^= 1u;
      const bool mok = umma::mbar_wait(umma::smem_u32(&mbar), mph, kWaitNs);
      mph ^= 1u;
      ok = __syncthreads_and(mok ? 1 : 0) != 0 && !s_abort;
      if (!ok) break;
      umma::tc_fence_after();
      // the weights are free again: stream in the next layer's (or the next tile's first) while the epilogue runs
      if (threadIdx.x == 0 && (l < kSurLayers - 1 || tile + gridDim.x < ntiles)) load_w((l + 1) % kSurLayers);
      for (int c0 = grp * kGroupCols; c0 < (grp + 1) * kGroupCols; c0 += 32) {
        float v[32];
        umma::tmem_ld32(trow + c0, v);
        const float4 *b4 = reinterpret_cast<const float4 *>(&s_bias[l][c0]);
        if (l < kSurLayers - 1) {
#pragma unroll
          for (int j = 0; j < 32; j += 8) {
            const float4 ba = b4[j / 4], bb = b4[j / 4 + 1];
            const float b[8] = {ba.x, ba.y, ba.z, ba.w, bb.x, bb.y, bb.z, bb.w};
            __align__(16) bf16 hb[8];
#pragma unroll
            for (int t = 0; t < 8; ++t) hb[t] = __float2bfloat16_rn(silu(v[j + t] + b[t]));
            *(uint4 *)(H + umma::sw128_offset(row, c0 + j, 128)) = *(const uint4 *)hb;
          }
        } else {
          const float4 *w0 = reinterpret_cast<const float4 *>(&s_wh[0][c0]);
          const float4 *w1 = reinterpret_cast<const float4 *>(&s_wh[1][c0]);
#pragma unroll
          for (int j = 0; j < 32; j += 4) {
            const float4 bq = b4[j / 4], m0 = w0[j / 4], m1 = w1[j / 4];
            const float b[4] = {bq.x, bq.y, bq.z, bq.w}, x0[4] = {m0.x, m0.y, m0.z, m0.w},
                        x1[4] = {m1.x, m1.y, m1.z, m1.w};
#pragma unroll
            for (int t = 0; t < 4; ++t) {
              const float h = silu(v[j + t] + b[t]);
              mu = fmaf(h, x0[t], mu);
              sl = fmaf(h, x1[t], sl);
            }
          }
        }
      }
      if (l < kSurLayers - 1) umma::fence_async_smem();
      umma::tc_fence_before();
      __syncthreads();
    }
    if (!ok) break;
    s_head[grp][row][0] = mu;
    s_head[grp][row][1] = sl;
    __syncthreads();
    if (grp == 0) {  // whole warps
      float m = s_bh[0], s = s_bh[1];
#pragma unroll
      for (int k = 0; k < kInferGroups; ++k) {
        m += s_head[k][row][0];
        s += s_head[k][row][1];
      }
      s = fminf(fmaxf(s, -12.0f), 4.0f);
      const float T = md.log_out ? md.t_shift + md.t_scale * expf(m) : md.t_shift + md.t_scale * m;
      const float e = md.log_out ? 2.0f * (T - md.t_shift) * expf(s) : 2.0f * md.t_scale * expf(s);
      if (SRC == kSrcArray) {
        if (valid) {
          a.T[qi] = T;
          a.err[qi] = e;
        }
      } else {
        const bool near = valid && fabsf(T - a.job.t_liq) < a.job.band;
        const bool fb = near && e > a.job.thresh;
        if (valid) {
          double out = (double)T;
          if (fb) out = scan_field(a.job.src, nx, ny, nz, frame_time(a.job, f));
          a.job.ring[(int64_t)(f % a.job.slots) * a.job.nnodes + node] = out;
        }
        const unsigned nv = __popc(__ballot_sync(0xffffffffu, valid));
        const unsigned nn = __popc(__ballot_sync(0xffffffffu, near));
        const unsigned nfb = __popc(__ballot_sync(0xffffffffu, fb));
        if (lane == 0) {
          if (nv) atomicAdd(&a.job.counters[0], (unsigned long long)nv);
          if (nn) atomicAdd(&a.job.counters[1], (unsigned long long)nn);
          if (nfb) atomicAdd(&a.job.counters[2], (unsigned long long)nfb);
        }
      }
    }
    __syncthreads();
  }
  if (!ok && threadIdx.x == 0) atomicCAS(a.error, 0, kErrWait);
  umma::tc_fence_before();
  __syncthreads();
  if (warp == 0) umma::tmem_free(tmem, 256);
}

}  // namespace sur
}  // namespace amca

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
namespace amca {
namespace sur {

#define SCK(call)                                                                                       \
  do {                                                                                                  \
    cudaError_t e_ = (call);                                                                            \
    if (e_ != cudaSuccess) throw std::runtime_error(std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    void *p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  });
  if (!fn) throw std::runtime_error("cuTensorMapEncodeTiled is not available");
  return fn;
}

// Tensor map of a row-major [rows x cols] bf16 matrix read in boxes of 64
// columns x box_rows rows with the 128-byte swizzle.
CUtensorMap tmap_bf16(const void *base, int64_t rows, int64_t cols, int box_rows) {
  if (cols % 64 != 0 || box_rows > 256 || ((uintptr_t)base & 15) != 0)
    throw std::invalid_argument("tensor map: columns must be a multiple of 64 and the base 16-byte aligned");
  CUtensorMap m;
  const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
  const cuuint32_t box[2] = {64, (cuuint32_t)box_rows};
  const cuuint32_t es[2] = {1, 1};
  const CUresult r = encode_fn()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box,
                                 es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                 CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw std::runtime_error("cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return m;
}

template <int EPI>
void launch_gemm(const CUtensorMap &tA, const CUtensorMap &tB, GemmArgs a, int splits, cudaStream_t s) {
  const size_t smem = (size_t)kStages * (16384 + (size_t)a.N * 128) + 1024;
  SCK(cudaFuncSetAttribute(mlp_gemm_kernel<EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (a.M % 128 || (a.N != 128 && a.N != 256) || a.K % (64 * splits))
    throw std::invalid_argument("layer GEMM: M must be a multiple of 128, N 128 or 256, K a multiple of 64 x splits");
  a.kb_per_split = a.K / 64 / splits;
  mlp_gemm_kernel<EPI><<<dim3(a.M / 128, 1, splits), 256, smem, s>>>(tA, tB, a);
  SCK(cudaGetLastError());
}

int grid_1d(int64_t n, int threads = 256) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + threads - 1) / threads, 152 * 16));
}

uint64_t gcd64(uint64_t a, uint64_t b) {
  while (b) {
    const uint64_t t = a % b;
    a = b;
    b = t;
  }
  return a;
}

}  // namespace sur

// One thermal model on one device: parameters, Adam state, the training set
// and the per-batch buffers of a training step.
struct ThermalModel {
  using bf16 = __nv_bfloat16;
  int device = 0;
  cudaStream_t stream = nullptr;
  SurParamLayout L;
  sur::DataSpec data{};
  float fourier_h[kSurFreq * kSurIn];
  float in_shift[kSurIn], in_scale[kSurIn], t_shift = 0, t_scale = 1;
  // device
  float *fourier = nullptr, *p = nullptr, *m1 = nullptr, *m2 = nullptr, *g = nullptr;
  bf16 *Wb[kSurLayers] = {}, *Wtb[kSurLayers] = {};
  int *err = nullptr;
  unsigned long long *counters = nullptr;
  float *ds_raw = nullptr, *ds_target = nullptr;
  int64_t ds_n = 0;
  int64_t adam_t = 0;
  int64_t seen = 0;
  // batch buffers
  int64_t nb = 0;
  int splits = 1;
  float *braw = nullptr, *by = nullptr, *pred = nullptr, *dpred = nullptr, *loss = nullptr, *partial = nullptr;
  bf16 *E = nullptr, *Et = nullptr, *Z[kSurLayers] = {}, *Hr[kSurLayers] = {}, *Ht[kSurLayers + 1] = {};
  bf16 *dZ[kSurLayers] = {}, *dZt[kSurLayers] = {};
  CUtensorMap tmA_fwd[kSurLayers], tmB_fwd[kSurLayers], tmA_dw[kSurLayers], tmB_dw[kSurLayers], tmA_dh[kSurLayers],
      tmB_dh[kSurLayers];
  std::vector<void *> allocs, batch_allocs;

  template <typename T>
  T *alloc(size_t n) {
    void *q = nullptr;
    SCK(cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T)));
    allocs.push_back(q);
    return (T *)q;
  }
  template <typename T>
  T *balloc(size_t n) {
    void *q = nullptr;
    SCK(cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T)));
    batch_allocs.push_back(q);
    return (T *)q;
  }
  ~ThermalModel() {
    if (stream) cudaStreamSynchronize(stream);
    for (void *q : batch_allocs) cudaFree(q);
    for (void *q : allocs) cudaFree(q);
    if (stream) cudaStreamDestroy(stream);
  }

  SurModelDev dev() const {
    SurModelDev d{};
    d.fourier = fourier;
    d.p = p;
    for (int l = 0; l < kSurLayers; ++l) d.Wb[l] = Wb[l];
    for (int i = 0; i < kSurIn; ++i) {
      d.in_shift[i] = in_shift[i];
      d.in_scale[i] = in_scale[i];
    }
    d.t_shift = t_shift;
    d.t_scale = t_scale;
    d.log_out = data.log_out;
    return d;
  }
  sur::AdamArgs adam_args() const {
    sur::AdamArgs a{};
    a.p = p;
    a.m = m1;
    a.v = m2;
    a.g = g;
    a.n = L.total;
    for (int l = 0; l < kSurLayers; ++l) {
      a.Wb[l] = Wb[l];
      a.Wtb[l] = Wtb[l];
      a.Woff[l] = L.W[l];
    }
    return a;
  }
  void check_error() {
    int e = 0;
    SCK(cudaMemcpyAsync(&e, err, sizeof e, cudaMemcpyDeviceToHost, stream));
    SCK(cudaStreamSynchronize(stream));
    if (e) throw std::runtime_error("thermal model kernel: a bounded wait ran out");
  }
  void refresh_bf16() {
    sur::refresh_bf16_kernel<<<sur::grid_1d(L.total), 256, 0, stream>>>(adam_args());
    SCK(cudaGetLastError());
  }

  ThermalModel(int dev_id, const sur::DataSpec &ds, double fourier_sigma, double fourier_sigma_pv)
      : device(dev_id), data(ds) {
    SCK(cudaSetDevice(device));
    SCK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    // input normalisation: the window's offsets and the power / speed ranges to [-1, 1]
    for (int a = 0; a < 3; ++a) {
      in_shift[a] = (float)(0.5 * (ds.win_lo[a] + ds.win_hi[a]));
      in_scale[a] = (float)(2.0 / (ds.win_hi[a] - ds.win_lo[a]));
    }
    in_shift[3] = (float)(0.5 * (ds.p_lo + ds.p_hi));
    in_scale[3] = (float)(2.0 / (ds.p_hi - ds.p_lo));
    in_shift[4] = (float)(0.5 * (ds.v_lo + ds.v_hi));
    in_scale[4] = (float)(2.0 / (ds.v_hi - ds.v_lo));
    t_shift = ds.t_shift;
    t_scale = ds.t_scale;
    // Fourier matrix: normal draws (Box-Muller on counter-based uniforms) times
    // sigma (offsets) or sigma_pv (power, speed)
    for (int i = 0; i < kSurFreq * kSurIn; ++i) {
      const double u1 = std::max(sur::uniform01(ds.seed, 100, (uint64_t)i), 1e-300);
      const double u2 = sur::uniform01(ds.seed, 101, (uint64_t)i);
      const double sig = (i % kSurIn) < 3 ? fourier_sigma : fourier_sigma_pv;
      fourier_h[i] = (float)(sig * std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2));
    }
    // weights: Xavier-uniform from the seed, biases zero; head small, log-error bias -2
    std::vector<float> ph((size_t)L.total, 0.0f);
    for (int l = 0; l < kSurLayers; ++l) {
      const int K = SurParamLayout::in_dim(l);
      const double bound = std::sqrt(6.0 / (K + kSurHid));
      for (int64_t i = 0; i < (int64_t)kSurHid * K; ++i)
        ph[L.W[l] + i] = (float)(bound * (2.0 * sur::uniform01(ds.seed, 200 + l, (uint64_t)i) - 1.0));
    }
    const double hb = 0.1 * std::sqrt(6.0 / (kSurHid + kSurOut));
    for (int64_t i = 0; i < (int64_t)kSurOut * kSurHid; ++i)
      ph[L.Wh + i] = (float)(hb * (2.0 * sur::uniform01(ds.seed, 300, (uint64_t)i) - 1.0));
    ph[L.bh + 1] = -2.0f;
    fourier = alloc<float>(kSurFreq * kSurIn);
    p = alloc<float>(L.total);
    m1 = alloc<float>(L.total);
    m2 = alloc<float>(L.total);
    g = alloc<float>(L.total);
    for (int l = 0; l < kSurLayers; ++l) {
      const int K = SurParamLayout::in_dim(l);
      Wb[l] = alloc<bf16>((size_t)kSurHid * K);
      if (l > 0) Wtb[l] = alloc<bf16>((size_t)kSurHid * K);
    }
    err = alloc<int>(1);
    counters = alloc<unsigned long long>(4);
    SCK(cudaMemcpyAsync(fourier, fourier_h, sizeof fourier_h, cudaMemcpyHostToDevice, stream));
    set_params(ph.data());
    SCK(cudaMemsetAsync(err, 0, sizeof(int), stream));
    SCK(cudaStreamSynchronize(stream));
  }

  void set_params(const float *host) {
    SCK(cudaMemcpyAsync(p, host, (size_t)L.total * 4, cudaMemcpyHostToDevice, stream));
    SCK(cudaMemsetAsync(m1, 0, (size_t)L.total * 4, stream));
    SCK(cudaMemsetAsync(m2, 0, (size_t)L.total * 4, stream));
    adam_t = 0;
    refresh_bf16();
    SCK(cudaStreamSynchronize(stream));
  }
  void get_params(float *host) {
    SCK(cudaMemcpyAsync(host, p, (size_t)L.total * 4, cudaMemcpyDeviceToHost, stream));
    SCK(cudaStreamSynchronize(stream));
  }

  // Per-batch buffers and tensor maps for batches of n rows (n a multiple of 128).
  void set_batch(int64_t n) {
    if (n == nb) return;
    if (n <= 0 || n % 128) throw std::invalid_argument("batch size must be a positive multiple of 128");
    SCK(cudaStreamSynchronize(stream));
    for (void *q : batch_allocs) cudaFree(q);
    batch_allocs.clear();
    nb = 0;
    const int64_t kblocks = n / 64;
    // split-K of the weight-gradient GEMMs: at most 64 splits of at least 8 K blocks
    splits = 1;
    while (splits < 64 && kblocks % (splits * 2) == 0 && kblocks / (splits * 2) >= 8) splits *= 2;
    braw = balloc<float>((size_t)n * kSurIn);
    by = balloc<float>((size_t)n);
    pred = balloc<float>((size_t)n * 2);
    dpred = balloc<float>((size_t)n * 2);
    loss = balloc<float>((size_t)n);
    partial = balloc<float>((size_t)splits * kSurHid * kSurHid);
    E = balloc<bf16>((size_t)n * kSurEnc);
    Et = balloc<bf16>((size_t)n * kSurEnc);
    Ht[0] = Et;
    for (int l = 0; l < kSurLayers; ++l) {
      Z[l] = balloc<bf16>((size_t)n * kSurHid);
      Hr[l] = balloc<bf16>((size_t)n * kSurHid);  // Hr[l] = H_{l+1} rows
      Ht[l + 1] = balloc<bf16>((size_t)n * kSurHid);
      dZ[l] = balloc<bf16>((size_t)n * kSurHid);
      dZt[l] = balloc<bf16>((size_t)n * kSurHid);
    }
    for (int l = 0; l < kSurLayers; ++l) {
      const int K = SurParamLayout::in_dim(l);
      // forward: A = layer input rows [n x K], B = W_l [256 x K]
      tmA_fwd[l] = sur::tmap_bf16(l == 0 ? (const void *)E : (const void *)Hr[l - 1], n, K, 128);
      tmB_fwd[l] = sur::tmap_bf16(Wb[l], kSurHid, K, 256);
      // weight gradient: A = dZ_l^T [256 x n], B = input^T [K x n]
      tmA_dw[l] = sur::tmap_bf16(dZt[l], kSurHid, n, 128);
      tmB_dw[l] = sur::tmap_bf16(Ht[l], K, n, K);
      // input gradient (l >= 1): A = dZ_l [n x 256], B = W_l^T [K x 256]
      if (l > 0) {
        tmA_dh[l] = sur::tmap_bf16(dZ[l], n, kSurHid, 128);
        tmB_dh[l] = sur::tmap_bf16(Wtb[l], K, kSurHid, 256);
      }
    }
    nb = n;
  }

  // Forward and backward over the batch in braw / by; gradients into g.
  void forward_backward() {
    using namespace sur;
    const int64_t n = nb;
    const SurModelDev md = dev();
    SCK(cudaMemsetAsync(err, 0, sizeof(int), stream));
    encode_kernel<<<grid_1d(n * kSurFreq), 256, 0, stream>>>(md, braw, n, n, E, Et);
    SCK(cudaGetLastError());
    for (int l = 0; l < kSurLayers; ++l) {
      GemmArgs a{};
      a.M = (int)n;
      a.N = kSurHid;
      a.K = SurParamLayout::in_dim(l);
      a.bias = p + L.b[l];
      a.error = err;
      if (l < kSurLayers - 1) {
        a.z_row = Z[l];
        a.out_row = Hr[l];
        a.out_t = Ht[l + 1];
        launch_gemm<kEpiFwd>(tmA_fwd[l], tmB_fwd[l], a, 1, stream);
      } else {
        a.head_t = Ht[l + 1];
        a.out_row = dZ[l];
        a.out_t = dZt[l];
        a.Wh = p + L.Wh;
        a.bh = p + L.bh;
        a.target = by;
        a.pred = pred;
        a.dpred = dpred;
        a.loss = loss;
        a.inv_batch = 1.0f / (float)n;
        a.lambda_s = 0.1f;
        launch_gemm<kEpiHead>(tmA_fwd[l], tmB_fwd[l], a, 1, stream);
      }
    }
    head_grad_kernel<<<kSurHid + 1, 256, 0, stream>>>(Ht[kSurLayers], dpred, n, kSurHid, g + L.Wh, g + L.bh);
    SCK(cudaGetLastError());
    for (int l = kSurLayers - 1; l >= 0; --l) {
      const int K = SurParamLayout::in_dim(l);
      row_sum_kernel<<<kSurHid, 256, 0, stream>>>(dZt[l], n, g + L.b[l]);
      SCK(cudaGetLastError());
      GemmArgs w{};
      w.M = kSurHid;
      w.N = K;
      w.K = (int)n;
      w.partial = partial;
      w.error = err;
      launch_gemm<kEpiPartial>(tmA_dw[l], tmB_dw[l], w, splits, stream);
      reduce_partials_kernel<<<grid_1d((int64_t)kSurHid * K), 256, 0, stream>>>(partial, splits,
                                                                                 (int64_t)kSurHid * K, g + L.W[l]);
      SCK(cudaGetLastError());
      if (l > 0) {
        GemmArgs b{};
        b.M = (int)n;
        b.N = K;
        b.K = kSurHid;
        b.z_in = Z[l - 1];
        b.out_row = l > 1 ? dZ[l - 1] : nullptr;
        b.out_t = dZt[l - 1];
        b.error = err;
        launch_gemm<kEpiBwd>(tmA_dh[l], tmB_dh[l], b, 1, stream);
      }
    }
  }

  void adam(float lr) {
    ++adam_t;
    sur::AdamArgs a = adam_args();
    a.lr = lr;
    a.beta1 = 0.9f;
    a.beta2 = 0.999f;
    a.eps = 1e-8f;
    a.bc1 = (float)(1.0 - std::pow(0.9, (double)adam_t));
    a.bc2 = (float)(1.0 - std::pow(0.999, (double)adam_t));
    sur::adam_kernel<<<sur::grid_1d(L.total), 256, 0, stream>>>(a);
    SCK(cudaGetLastError());
  }

  void make_dataset(int64_t n) {
    if (n == ds_n) return;
    if (n <= 0) throw std::invalid_argument("training set size must be positive");
    SCK(cudaStreamSynchronize(stream));
    if (ds_raw) {
      cudaFree(ds_raw);
      cudaFree(ds_target);
      allocs.erase(std::remove(allocs.begin(), allocs.end(), (void *)ds_raw), allocs.end());
      allocs.erase(std::remove(allocs.begin(), allocs.end(), (void *)ds_target), allocs.end());
    }
    ds_raw = alloc<float>((size_t)n * kSurIn);
    ds_target = alloc<float>((size_t)n);
    ds_n = n;
    sur::make_data_kernel<<<sur::grid_1d(n), 256, 0, stream>>>(data, 0, n, ds_raw, ds_target);
    SCK(cudaGetLastError());
  }
};

// FrameJob of a scan: node grid and source from amca_scan.
sur::FrameJob scan_job(const amca_scan &p) {
  sur::FrameJob j{};
  for (int a = 0; a < 3; ++a) {
    j.origin[a] = p.origin[a];
    j.nodes[a] = p.nodes[a];
  }
  j.spacing = p.spacing;
  j.length_scale = p.length_scale;
  j.frame_dt = p.frame_dt;
  j.time_scale = p.time_scale;
  j.nnodes = (int64_t)p.nodes[0] * p.nodes[1] * p.nodes[2];
  ScanSource &s = j.src;
  s.power = p.power;
  s.absorptivity = p.absorptivity;
  s.speed = p.speed;
  s.conductivity = p.conductivity;
  s.diffusivity = p.diffusivity;
  s.t0 = p.t0;
  s.t_cap = p.t_cap;
  s.x_start = p.x_start;
  s.x_turn = p.x_turn;
  s.y_line = p.y_line;
  s.z_top = p.z_top;
  s.hatch = p.hatch;
  s.track_time = p.track_time;
  s.ntracks = p.ntracks;
  return j;
}

void check_scan(const amca_scan &p) {
  for (int a = 0; a < 3; ++a)
    if (p.nodes[a] < 2) throw std::invalid_argument("scan: at least 2 nodes per axis");
  if (p.frames < 2) throw std::invalid_argument("scan: at least two frames");
  if (!(p.spacing > 0) || !(p.length_scale > 0) || !(p.frame_dt > 0) || !(p.time_scale > 0))
    throw std::invalid_argument("scan: spacing, length_scale, frame_dt and time_scale must be positive");
  if (p.ntracks > 1 && !(p.track_time > 0)) throw std::invalid_argument("scan: track_time must be positive");
}

// Frames of job.f0 .. job.f0 + job.nf - 1 into the job's ring: the FE field
// of the scan (model == nullptr) or the model with its fallback.
void produce_frames(ThermalModel *model, sur::FrameJob job, cudaStream_t s) {
  using namespace sur;
  const int64_t total = job.nnodes * job.nf;
  if (!model) {
    scan_frames_kernel<<<grid_1d(total), 256, 0, s>>>(job);
    SCK(cudaGetLastError());
    return;
  }
  fill_frames_kernel<<<grid_1d(total), 256, 0, s>>>(job);
  SCK(cudaGetLastError());
  const double h = job.spacing * job.length_scale;
  for (int a = 0; a < 3; ++a) {
    job.win_lo[a] = model->data.win_lo[a];
    job.win_hi[a] = model->data.win_hi[a];
    job.box[a] = (int)std::ceil((job.win_hi[a] - job.win_lo[a]) / h) + 2;
  }
  if (!job.counters) job.counters = model->counters;
  InferArgs ia{};
  ia.nq = (int64_t)job.box[0] * job.box[1] * job.box[2] * job.nf;
  ia.job = job;
  ia.error = model->err;
  CUtensorMap tw[kSurLayers];
  for (int l = 0; l < kSurLayers; ++l) tw[l] = tmap_bf16(model->Wb[l], kSurHid, SurParamLayout::in_dim(l), 256);
  int sms = 0;
  SCK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, model->device));
  SCK(cudaFuncSetAttribute(mlp_infer_kernel<kSrcFrames>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kInferSmem));
  const int64_t tiles = (ia.nq + 127) / 128;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(tiles, sms));
  mlp_infer_kernel<kSrcFrames><<<grid, kInferThreads, kInferSmem, s>>>(tw[0], tw[1], tw[2], tw[3], model->dev(), ia);
  SCK(cudaGetLastError());
}

}  // namespace amca

struct amca_thermal {
  std::string err;
  std::unique_ptr<amca::ThermalModel> m;
};

namespace {

template <typename F>
int tguard(amca_thermal *h, F &&f) {
  try {
    f();
    if (h) h->err.clear();
    return AMCA_OK;
  } catch (const std::invalid_argument &e) {
    if (h) h->err = e.what();
    return AMCA_ERR_ARG;
  } catch (const std::exception &e) {
    if (h) h->err = e.what();
    return AMCA_ERR_CUDA;
  }
}

struct DeviceBuffers {
  std::vector<void *> p;
  void *get(size_t bytes) {
    void *q = nullptr;
    SCK(cudaMalloc(&q, std::max<size_t>(bytes, 1)));
    p.push_back(q);
    return q;
  }
  ~DeviceBuffers() {
    for (void *q : p) cudaFree(q);
  }
};

}  // namespace

namespace amca {

ThermalModel *thermal_model_of(void *handle) { return handle ? ((amca_thermal *)handle)->m.get() : nullptr; }

void fill_scan_frames(const amca_scan *scan, ThermalModel *model, double t_liq, double band, double thresh, int f0,
                      int nf, double *ring, int slots, unsigned long long *counters, cudaStream_t s) {
  sur::FrameJob job = scan_job(*scan);
  job.f0 = f0;
  job.nf = nf;
  job.ring = ring;
  job.slots = slots;
  job.t_liq = (float)t_liq;
  job.band = (float)band;
  job.thresh = (float)thresh;
  job.counters = counters;
  produce_frames(model, job, s);
}

}  // namespace amca

extern "C" {

int amca_thermal_create(int device, const amca_thermal_spec *spec, amca_thermal **out) {
  if (!spec || !out) return AMCA_ERR_ARG;
  *out = nullptr;
  std::unique_ptr<amca_thermal> h(new amca_thermal);
  const int rc = tguard(h.get(), [&] {
    if (!(spec->power_hi > spec->power_lo) || !(spec->speed_hi > spec->speed_lo) || !(spec->t_scale > 0))
      throw std::invalid_argument("amca_thermal_create: empty power or speed range, or t_scale <= 0");
    if (spec->log_output && !(spec->t_shift < spec->t0))
      throw std::invalid_argument("amca_thermal_create: a log output needs t_shift below t0");
    for (int a = 0; a < 3; ++a)
      if (!(spec->window_hi[a] > spec->window_lo[a]) || !(spec->near_hi[a] > spec->near_lo[a]))
        throw std::invalid_argument("amca_thermal_create: empty window or melt-pool box");
    amca::sur::DataSpec ds{};
    ds.seed = spec->seed;
    ds.p_lo = spec->power_lo;
    ds.p_hi = spec->power_hi;
    ds.v_lo = spec->speed_lo;
    ds.v_hi = spec->speed_hi;
    for (int a = 0; a < 3; ++a) {
      ds.win_lo[a] = spec->window_lo[a];
      ds.win_hi[a] = spec->window_hi[a];
      ds.near_lo[a] = spec->near_lo[a];
      ds.near_hi[a] = spec->near_hi[a];
    }
    ds.near = spec->near_fraction;
    ds.shell = spec->shell_fraction;
    ds.shell_lo = spec->shell_lo;
    ds.shell_hi = spec->shell_hi;
    if (!(ds.near >= 0) || !(ds.shell >= 0) || ds.near + ds.shell > 1.0)
      throw std::invalid_argument("amca_thermal_create: near_fraction + shell_fraction must lie in [0, 1]");
    ds.src.absorptivity = spec->absorptivity;
    ds.src.conductivity = spec->conductivity;
    ds.src.diffusivity = spec->diffusivity;
    ds.src.t0 = spec->t0;
    ds.src.t_cap = spec->t_cap;
    ds.src.ntracks = 1;
    ds.t_shift = (float)spec->t_shift;
    ds.t_scale = (float)spec->t_scale;
    ds.log_out = spec->log_output ? 1 : 0;
    h->m.reset(new amca::ThermalModel(device, ds, spec->fourier_sigma, spec->fourier_sigma_pv));
  });
  if (rc == AMCA_OK) *out = h.release();
  return rc;
}

int amca_thermal_train(amca_thermal *h, int64_t samples, int steps, int batch, double lr_max, double lr_min,
                       amca_thermal_train_stats *st) {
  if (!h || steps < 0) return AMCA_ERR_ARG;
  return tguard(h, [&] {
    amca::ThermalModel &m = *h->m;
    SCK(cudaSetDevice(m.device));
    m.make_dataset(samples);
    m.set_batch(batch);
    uint64_t a = 2654435761ull;
    while (amca::sur::gcd64(a, (uint64_t)samples) != 1) a += 2;
    DeviceBuffers tmp;
    double *acc = (double *)tmp.get(2 * sizeof(double));
    SCK(cudaMemsetAsync(acc, 0, 2 * sizeof(double), m.stream));
    const int edge = std::max(1, steps / 20);
    const int warm = std::max(1, steps / 50);
    SCK(cudaStreamSynchronize(m.stream));
    const auto t0 = std::chrono::steady_clock::now();
    for (int s = 0; s < steps; ++s) {
      amca::sur::gather_batch_kernel<<<amca::sur::grid_1d(m.nb), 256, 0, m.stream>>>(
          m.ds_raw, m.ds_target, m.ds_n, m.seen % m.ds_n, m.nb, a, m.braw, m.by);
      SCK(cudaGetLastError());
      m.seen += m.nb;
      m.forward_backward();
      const double frac = s < warm ? (double)(s + 1) / warm : (double)(s - warm) / std::max(1, steps - warm);
      const double lr = s < warm ? lr_max * frac : lr_min + 0.5 * (lr_max - lr_min) * (1.0 + std::cos(M_PI * frac));
      m.adam((float)lr);
      if (s < edge || s >= steps - edge)
        amca::sur::accum_loss_kernel<<<64, 256, 0, m.stream>>>(m.loss, m.nb, acc + (s < edge ? 0 : 1));
    }
    SCK(cudaStreamSynchronize(m.stream));
    const auto t1 = std::chrono::steady_clock::now();
    m.check_error();
    double hacc[2] = {0, 0};
    SCK(cudaMemcpy(hacc, acc, sizeof hacc, cudaMemcpyDeviceToHost));
    if (st) {
      st->steps = steps;
      st->samples_seen = m.seen;
      st->first_loss = hacc[0] / ((double)edge * m.nb);
      st->last_loss = hacc[1] / ((double)edge * m.nb);
      st->ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    }
  });
}

int amca_thermal_eval(amca_thermal *h, const float *raw, int64_t n, float *T, float *err) {
  if (!h || n < 0 || (n > 0 && (!raw || !T || !err))) return AMCA_ERR_ARG;
  return tguard(h, [&] {
    using namespace amca::sur;
    amca::ThermalModel &m = *h->m;
    SCK(cudaSetDevice(m.device));
    if (n == 0) return;
    DeviceBuffers tmp;
    float *d_raw = (float *)tmp.get((size_t)n * amca::kSurIn * 4);
    float *d_T = (float *)tmp.get((size_t)n * 4);
    float *d_e = (float *)tmp.get((size_t)n * 4);
    SCK(cudaMemcpyAsync(d_raw, raw, (size_t)n * amca::kSurIn * 4, cudaMemcpyHostToDevice, m.stream));
    SCK(cudaMemsetAsync(m.err, 0, sizeof(int), m.stream));
    InferArgs ia{};
    ia.nq = n;
    ia.raw = d_raw;
    ia.T = d_T;
    ia.err = d_e;
    ia.error = m.err;
    CUtensorMap tw[amca::kSurLayers];
    for (int l = 0; l < amca::kSurLayers; ++l)
      tw[l] = tmap_bf16(m.Wb[l], amca::kSurHid, amca::SurParamLayout::in_dim(l), 256);
    int sms = 0;
    SCK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, m.device));
    SCK(cudaFuncSetAttribute(mlp_infer_kernel<kSrcArray>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kInferSmem));
    const int64_t tiles = (n + 127) / 128;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(tiles, sms));
    mlp_infer_kernel<kSrcArray><<<grid, kInferThreads, kInferSmem, m.stream>>>(tw[0], tw[1], tw[2], tw[3], m.dev(), ia);
    SCK(cudaGetLastError());
    SCK(cudaMemcpyAsync(T, d_T, (size_t)n * 4, cudaMemcpyDeviceToHost, m.stream));
    SCK(cudaMemcpyAsync(err, d_e, (size_t)n * 4, cudaMemcpyDeviceToHost, m.stream));
    SCK(cudaStreamSynchronize(m.stream));
    m.check_error();
  });
}

int amca_thermal_gradients(amca_thermal *h, const float *raw, const float *target, int64_t n, float *grad,
                           float *pred) {
  if (!h || !raw || !target || !grad || n <= 0) return AMCA_ERR_ARG;
  return tguard(h, [&] {
    amca::ThermalModel &m = *h->m;
    SCK(cudaSetDevice(m.device));
    m.set_batch(n);
    SCK(cudaMemcpyAsync(m.braw, raw, (size_t)n * amca::kSurIn * 4, cudaMemcpyHostToDevice, m.stream));
    SCK(cudaMemcpyAsync(m.by, target, (size_t)n * 4, cudaMemcpyHostToDevice, m.stream));
    m.forward_backward();
    SCK(cudaMemcpyAsync(grad, m.g, (size_t)m.L.total * 4, cudaMemcpyDeviceToHost, m.stream));
    if (pred) SCK(cudaMemcpyAsync(pred, m.pred, (size_t)n * 2 * 4, cudaMemcpyDeviceToHost, m.stream));
    SCK(cudaStreamSynchronize(m.stream));
    m.check_error();
  });
}

int64_t amca_thermal_param_count(void) { return amca::SurParamLayout().total; }

int amca_thermal_get_params(amca_thermal *h, float *params) {
  if (!h || !params) return AMCA_ERR_ARG;
  return tguard(h, [&] {
    SCK(cudaSetDevice(h->m->device));
    h->m->get_params(params);
  });
}

int amca_thermal_set_params(amca_thermal *h, const float *params) {
  if (!h || !params) return AMCA_ERR_ARG;
  return tguard(h, [&] {
    SCK(cudaSetDevice(h->m->device));
    h->m->set_params(params);
  });
}

int amca_thermal_get_encoding(amca_thermal *h, float *fourier, float *in_shift, float *in_scale, float *t_shift,
                              float *t_scale, int32_t *log_output) {
  if (!h) return AMCA_ERR_ARG;
  const amca::ThermalModel &m = *h->m;
  if (fourier) memcpy(fourier, m.fourier_h, sizeof m.fourier_h);
  if (in_shift) memcpy(in_shift, m.in_shift, sizeof m.in_shift);
  if (in_scale) memcpy(in_scale, m.in_scale, sizeof m.in_scale);
  if (t_shift) *t_shift = m.t_shift;
  if (t_scale) *t_scale = m.t_scale;
  if (log_output) *log_output = m.data.log_out;
  return AMCA_OK;
}

int amca_thermal_frames(amca_thermal *h, const amca_scan *scan, int32_t f0, int32_t nf, double t_liq, double band,
                        double thresh, double *frames, double *fe, int64_t *counts) {
  if (!h || !scan || !frames || f0 < 0 || nf < 1) return AMCA_ERR_ARG;
  return tguard(h, [&] {
    amca::ThermalModel &m = *h->m;
    SCK(cudaSetDevice(m.device));
    amca::check_scan(*scan);
    amca::sur::FrameJob job = amca::scan_job(*scan);
    job.f0 = f0;
    job.nf = nf;
    job.slots = nf;
    job.t_liq = (float)t_liq;
    job.band = (float)band;
    job.thresh = (float)thresh;
    DeviceBuffers tmp;
    double *ring = (double *)tmp.get((size_t)nf * job.nnodes * 8);
    job.ring = ring;
    SCK(cudaMemsetAsync(m.counters, 0, 4 * sizeof(unsigned long long), m.stream));
    SCK(cudaMemsetAsync(m.err, 0, sizeof(int), m.stream));
    amca::produce_frames(&m, job, m.stream);
    // slot of frame f is f % nf: copy back in frame order
    auto fetch = [&](double *dst) {
      for (int k = 0; k < nf; ++k) {
        const int slot = (f0 + k) % nf;
        SCK(cudaMemcpyAsync(dst + (size_t)k * job.nnodes, ring + (size_t)slot * job.nnodes, job.nnodes * 8,
                            cudaMemcpyDeviceToHost, m.stream));
      }
    };
    fetch(frames);
    unsigned long long c[4] = {0, 0, 0, 0};
    SCK(cudaMemcpyAsync(c, m.counters, sizeof c, cudaMemcpyDeviceToHost, m.stream));
    if (fe) {
      amca::produce_frames(nullptr, job, m.stream);
      fetch(fe);
    }
    SCK(cudaStreamSynchronize(m.stream));
    m.check_error();
    if (counts)
      for (int i = 0; i < 3; ++i) counts[i] = (int64_t)c[i];
  });
}

const char *amca_thermal_last_error(const amca_thermal *h) { return h ? h->err.c_str() : "null handle"; }

void amca_thermal_destroy(amca_thermal *h) { delete h; }

}  // extern "C"
