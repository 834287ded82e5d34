// kmc_mlp.cu -- the learned pair-rate surrogate: training (forward + backward + Adam), inference
// and the table builder that turns the network into a KMC_TABLE_2D_SPECIES rate table.
//
// The network is tiny (4 -> 64 -> 64 -> 1, 4.6k parameters) and a 2M-sample epoch is ~55 GFLOP.
// Training runs its three 64-wide contractions per 128-sample chunk on the tensor cores (TF32
// warp MMAs with split operands, k_mlp_grad) and the rest on the CUDA cores; the weight gradients
// are summed per block in a fixed order, then across blocks in block order: training is
// deterministic.  Inference (k_mlp_predict, k_mlp_table) carries one sample per thread through
// the network in FP32 with the weights staged in shared memory (broadcast reads).
#include <cuda_bf16.h>

#include "../../include/cntkmc.h"
#include "kmc_internal.h"

namespace kmc {
namespace {

constexpr float kGeluK0 = 0.7978845608028654f;  // sqrt(2 / pi), GELU tanh form (Hendrycks & Gimpel)
constexpr float kGeluK1 = 0.044715f;
constexpr double kThetaScale = 1.2732395447351628;  // 4 / pi: theta in [0, pi/2] -> [0, 2]

// The network staged in shared memory as FP32 (the BF16 matrices widened exactly).
struct __align__(16) MlpSmem {
  float w1[kMlpH * 4];
  float b1[kMlpH];
  float w2[kMlpH * kMlpH];
  float b2[kMlpH];
  float w3[kMlpH];
  float b3[4];
  float e[2 * KMC_MAX_SPECIES * KMC_MAX_SPECIES];
};

__device__ __forceinline__ float widen(uint16_t b) { return __uint_as_float((uint32_t)b << 16); }

__device__ void stage(const MlpDev& m, MlpSmem& w) {
  for (int i = threadIdx.x; i < kMlpH * 4; i += blockDim.x) w.w1[i] = widen(m.wbf[kMlpOffW1 + i]);
  for (int i = threadIdx.x; i < kMlpH * kMlpH; i += blockDim.x) w.w2[i] = widen(m.wbf[kMlpOffW2 + i]);
  for (int i = threadIdx.x; i < kMlpH; i += blockDim.x) {
    w.b1[i] = m.master[kMlpOffB1 + i];
    w.b2[i] = m.master[kMlpOffB2 + i];
    w.w3[i] = widen(m.wbf[kMlpOffW3 + i]);
  }
  const int ne = 2 * m.n_species * m.n_species;
  for (int i = threadIdx.x; i < ne; i += blockDim.x) w.e[i] = m.master[kMlpOffE + i];
  if (threadIdx.x == 0) w.b3[0] = m.master[kMlpOffB3];
  __syncthreads();
}

__device__ __forceinline__ float gelu(float z, float& t) {
  t = tanhf(kGeluK0 * (z + kGeluK1 * z * z * z));
  return 0.5f * z * (1.f + t);
}
// The training kernel's GELU: tanh(u) = 1 - 2 / (1 + e^(2u)) with the hardware exponential and
// division (u clamped to [-9, 9], where tanh is +-1 in FP32), ~5e-7 absolute against tanhf; the
// network's outputs (k_mlp_predict, k_mlp_table) use tanhf.
__device__ __forceinline__ float gelu_train(float z, float& t) {
  const float u = fminf(fmaxf(kGeluK0 * (z + kGeluK1 * z * z * z), -9.f), 9.f);
  t = 1.f - __fdividef(2.f, 1.f + __expf(2.f * u));
  return 0.5f * z * (1.f + t);
}
__device__ __forceinline__ float gelu_grad(float z, float t) {
  return 0.5f * (1.f + t) + 0.5f * z * (1.f - t * t) * kGeluK0 * (1.f + 3.f * kGeluK1 * z * z);
}

__device__ __forceinline__ float layer1(const MlpSmem& w, int i, float x0, float x1, float x2, float x3) {
  float z = w.b1[i];
  z = fmaf(w.w1[4 * i], x0, z);
  z = fmaf(w.w1[4 * i + 1], x1, z);
  z = fmaf(w.w1[4 * i + 2], x2, z);
  return fmaf(w.w1[4 * i + 3], x3, z);
}

__device__ __forceinline__ float layer1_s(const float* w1, const float* b1, int i, float x0, float x1, float x2, float x3) {
  float z = b1[i];
  z = fmaf(w1[4 * i], x0, z);
  z = fmaf(w1[4 * i + 1], x1, z);
  z = fmaf(w1[4 * i + 2], x2, z);
  return fmaf(w1[4 * i + 3], x3, z);
}

// Layer-2 pre-activation of unit j: four independent partial sums (columns i mod 4), so a warp
// (one per scheduler at this kernel's occupancy) has four FMA chains in flight, not one.
__device__ __forceinline__ float row_dot(const MlpSmem& w, int j, const float (&a)[kMlpH]) {
  const float4* r = reinterpret_cast<const float4*>(w.w2 + j * kMlpH);
  float z0 = w.b2[j], z1 = 0.f, z2 = 0.f, z3 = 0.f;
#pragma unroll
  for (int q = 0; q < kMlpH / 4; ++q) {
    const float4 c = r[q];
    z0 = fmaf(c.x, a[4 * q], z0);
    z1 = fmaf(c.y, a[4 * q + 1], z1);
    z2 = fmaf(c.z, a[4 * q + 2], z2);
    z3 = fmaf(c.w, a[4 * q + 3], z3);
  }
  return (z0 + z1) + (z2 + z3);
}

// Network output (normalised log-rate) of one input.
__device__ float forward(const MlpSmem& w, float x0, float x1, int pair) {
  const float x2 = w.e[2 * pair], x3 = w.e[2 * pair + 1];
  float a1[kMlpH];
#pragma unroll
  for (int i = 0; i < kMlpH; ++i) {
    float t;
    a1[i] = gelu(layer1(w, i, x0, x1, x2, x3), t);
  }
  float y = w.b3[0];
  for (int j = 0; j < kMlpH; ++j) {
    float t;
    y = fmaf(w.w3[j], gelu(row_dot(w, j, a1), t), y);
  }
  return y;
}

__device__ __forceinline__ float dist_input(const MlpDev& m, double d) {
  return (float)(log(d / m.d_min) * m.inv_span - 1.0);
}
__device__ __forceinline__ float angle_input(double theta) { return (float)(theta * kThetaScale - 1.0); }

__global__ void k_mlp_samples(MlpDev m, const double* dist, const double* theta, const int32_t* pair,
                              const double* log_rate, int64_t n, float4* out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = make_float4(dist_input(m, dist[i]), angle_input(theta[i]), __int_as_float(pair[i]),
                       (float)((log_rate[i] - m.log_mean) / m.log_scale));
}

__global__ void k_mlp_bf16(const float* master, uint16_t* wbf, int32_t n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) wbf[i] = __bfloat16_as_ushort(__float2bfloat16_rn(master[i]));
}

// ---------------------------------------------------------------- tensor-core gradient kernel
// The three 64-wide contractions of a 128-sample chunk run on the tensor cores as warp MMAs
// (mma.sync m16n8k8, TF32 operands, FP32 accumulation):
//   Z2 = A1 W2^T      (128 x 64 x 64)  layer-2 pre-activations
//   G1 = D2 W2        (128 x 64 x 64)  gradient of the layer-1 outputs
//   dW2 += D2^T A1    (64 x 64 x 128)  layer-2 weight gradient, summed over the chunk's samples
// TF32 keeps 10 mantissa bits, so every activation and delta is split into hi + lo TF32 parts
// (hi = x rounded to TF32, lo = the rest rounded to TF32) and a product a b is formed as
// a_hi b + a_lo b, or a_hi b_hi + a_hi b_lo + a_lo b_hi when both sides are activations: the
// result carries ~22 significant bits, the FP32 SIMT sums' accuracy.  The BF16 weight entries are
// exact in TF32 and need no split.  Everything else (layer 1, GELU, the output layer, the small
// gradients) stays in FP32 on the CUDA cores.
//
// A block of 8 warps takes a chunk of 128 samples: warp w owns samples 16w .. 16w + 15 (one
// 16-row tile) for the forward and backward passes, and rows 16 (w mod 4) .. + 15, columns
// 32 (w / 4) .. + 31 of dW2.  Fragment layouts (PTX ISA, mma.m16n8k8 .tf32), with
// g = lane / 4 and q = lane % 4: A (16 x 8, row-major) a0 (g, q), a1 (g + 8, q), a2 (g, q + 4),
// a3 (g + 8, q + 4); B (8 x 8) b0 (k = q, n = g), b1 (k = q + 4, n = g); C (16 x 8) c0 (g, 2q),
// c1 (g, 2q + 1), c2 (g + 8, 2q), c3 (g + 8, 2q + 1).  A thread therefore holds, in C layout,
// rows {g, g + 8} of its two tiles and columns 2q, 2q + 1 of each 8-column tile.
//
// Shared arrays read as fragments keep conflict-free strides: 68 words where a fragment walks
// rows at fixed column offsets q (bank 4g + q), 72 words where it walks columns (bank 8q + g).
// A1 and D2 are stored twice (68 for the row-major reads of the forward and backward passes,
// 72 for the transposed reads of the dW2 contraction).
constexpr int kS68 = 68, kS72 = 72;
constexpr int kGradThreads = 256;
constexpr int kGradWarps = kGradThreads / 32;
constexpr int kMT = kMlpChunk / (16 * kGradWarps);  // 16-row tiles per warp
struct __align__(16) WeightImage {
  float w2[kMlpH * kS68];    // W2[j][i] (row j: unit j)
  float w2t[kMlpH * kS68];   // W2^T[i][j]
  float w1[kMlpH * 4];
  float b1[kMlpH], b2[kMlpH], w3[kMlpH];
  float e[2 * KMC_MAX_SPECIES * KMC_MAX_SPECIES];
  float b3[4];
};
static_assert(sizeof(WeightImage) == kMlpImageFloats * sizeof(float), "image layout");
static_assert(sizeof(WeightImage) % 16 == 0, "image copied in 16-byte words");
struct __align__(16) GradSmem {
  WeightImage w;
  float a1[kMlpChunk * kS68];
  float a1t[kMlpChunk * kS72];
  float d2[kMlpChunk * kS68];
  float d2t[kMlpChunk * kS72];
  float x[kMlpChunk][4];     // inputs of the chunk's samples
  float dx[kMlpChunk][2];    // embedding-input gradients
  float err[kMlpChunk];      // squared errors
  float dy[kMlpChunk];       // output deltas
  int pair[kMlpChunk];       // pair index, -1 past the end
  // per-warp partial sums of the small gradients over the warp's samples (added in warp order)
  float w_w1[kGradWarps][kMlpH * 4];
  float w_b1[kGradWarps][kMlpH], w_b2[kGradWarps][kMlpH], w_w3[kGradWarps][kMlpH];
  float w_b3[kGradWarps];
  float emb[2][kMlpChunk];   // embedding gradients of the two sample halves
};

__device__ __forceinline__ uint32_t to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ void split_tf32(float x, uint32_t& hi, uint32_t& lo) {
  hi = to_tf32(x);
  lo = to_tf32(x - __uint_as_float(hi));
}
__device__ __forceinline__ void mma_tf32(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1) {
  asm("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// acc[mt][nt] += A[32w + 16 mt ..][0..64) B, A row-major in shared memory (stride 68, split into
// hi + lo), B[k][n] = bt[n * 68 + k] (TF32-exact weights)
__device__ __forceinline__ void warp_gemm_rows(float (&acc)[kMT][8][4], const float* __restrict__ a,
                                               const float* __restrict__ bt, int row0, int g, int q) {
#pragma unroll 1
  for (int ks = 0; ks < kMlpH / 8; ++ks) {
    uint32_t ah[kMT][4], al[kMT][4];
#pragma unroll
    for (int mt = 0; mt < kMT; ++mt) {
      const float* r0 = a + (row0 + 16 * mt + g) * kS68 + 8 * ks + q;
      split_tf32(r0[0], ah[mt][0], al[mt][0]);
      split_tf32(r0[8 * kS68], ah[mt][1], al[mt][1]);
      split_tf32(r0[4], ah[mt][2], al[mt][2]);
      split_tf32(r0[8 * kS68 + 4], ah[mt][3], al[mt][3]);
    }
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      const float* c0 = bt + (8 * nt + g) * kS68 + 8 * ks + q;
      const uint32_t b0 = __float_as_uint(c0[0]), b1 = __float_as_uint(c0[4]);
#pragma unroll
      for (int mt = 0; mt < kMT; ++mt) {
        mma_tf32(acc[mt][nt], ah[mt][0], ah[mt][1], ah[mt][2], ah[mt][3], b0, b1);
        mma_tf32(acc[mt][nt], al[mt][0], al[mt][1], al[mt][2], al[mt][3], b0, b1);
      }
    }
  }
}

// Gradient of sum_k (y_k - label_k)^2 / count over samples [first, first + count).  Block b takes
// chunks b, b + grid, ... of 128 samples and adds the chunk's gradients in a fixed order (MMA
// k-steps in sample order, warp partials in warp order); each block writes its partials to
// part[b][*], which k_mlp_update adds in block order: training is deterministic.
__global__ void __launch_bounds__(kGradThreads, 1)
    k_mlp_grad(MlpDev m, const float4* smp, int64_t first, int64_t count, float* part, double* part_loss,
               unsigned long long* step_ctr) {
  extern __shared__ __align__(16) unsigned char smem[];
  GradSmem& S = *reinterpret_cast<GradSmem*>(smem);
  const int t = threadIdx.x, lane = t & 31, w = t >> 5, g = lane >> 2, q = lane & 3;
  if (step_ctr && blockIdx.x == 0 && t == 0) atomicAdd(step_ctr, 1ull);
  // thread t < 128: its sample of the next chunk, loaded one chunk ahead
  const int64_t n_chunks = (count + kMlpChunk - 1) / kMlpChunk;
  auto load_sample = [&](int64_t c) {
    const int64_t k = c * kMlpChunk + t;
    return (t < kMlpChunk && c < n_chunks && k < count) ? smp[first + k] : make_float4(0.f, 0.f, 0.f, 0.f);
  };
  float4 sm_next = load_sample(blockIdx.x);
  {
    const float4* src = reinterpret_cast<const float4*>(m.image);
    float4* dst = reinterpret_cast<float4*>(&S.w);
    for (int i = t; i < (int)(sizeof(WeightImage) / 16); i += kGradThreads) dst[i] = src[i];
  }
  const int n_emb = 2 * m.n_species * m.n_species;
  for (int i = t; i < kGradWarps * kMlpH * 4; i += kGradThreads) (&S.w_w1[0][0])[i] = 0.f;
  for (int i = t; i < kGradWarps * kMlpH; i += kGradThreads) {
    (&S.w_b1[0][0])[i] = 0.f;
    (&S.w_b2[0][0])[i] = 0.f;
    (&S.w_w3[0][0])[i] = 0.f;
  }
  if (t < kGradWarps) S.w_b3[t] = 0.f;
  __syncthreads();
  const float scale = (float)(2.0 / (double)count);
  const int row0 = 16 * kMT * w;
  const int jt = w & 3, nt0 = 4 * (w >> 2);  // the warp's dW2 tile: rows 16 jt + {g, g + 8}
  float acc3[4][4];  // dW2 columns 8 (nt0 + n) + 2q + {0, 1}, summed over all chunks
#pragma unroll
  for (int nt = 0; nt < 4; ++nt)
#pragma unroll
    for (int e = 0; e < 4; ++e) acc3[nt][e] = 0.f;
  float acc_e = 0.f;      // embedding entry t & 127, samples of half t >> 7
  double acc_loss = 0.0;  // warp 0, lane 0
  for (int64_t c = blockIdx.x; c < n_chunks; c += gridDim.x) {
    // ---- inputs of the chunk (thread t < 128: sample t)
    const float4 sm = sm_next;
    sm_next = load_sample(c + gridDim.x);
    if (t < kMlpChunk) {
      const bool valid = c * kMlpChunk + t < count;
      const int pair = valid ? __float_as_int(sm.z) : 0;
      S.x[t][0] = sm.x;
      S.x[t][1] = sm.y;
      S.x[t][2] = S.w.e[2 * pair];
      S.x[t][3] = S.w.e[2 * pair + 1];
      S.pair[t] = valid ? pair : -1;
      S.dy[t] = sm.w;  // the label until the output delta replaces it
    }
    __syncthreads();
    // ---- layer 1 in C layout: rows r(mt, h) = row0 + 16 mt + g + 8 h, columns 8 nt + 2q + u.
    // Its GELU derivative waits in d2t (free until the layer-2 deltas), then in a1 (free once
    // the layer-2 contraction has read it), at the thread's own positions.
#pragma unroll
    for (int mt = 0; mt < kMT; ++mt)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int r = row0 + 16 * mt + g + 8 * h;
        const float x0 = S.x[r][0], x1 = S.x[r][1], x2 = S.x[r][2], x3 = S.x[r][3];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
          for (int u = 0; u < 2; ++u) {
            const int i = 8 * nt + 2 * q + u;
            const float z = layer1_s(S.w.w1, S.w.b1, i, x0, x1, x2, x3);
            float th;
            const float a = gelu_train(z, th);
            S.d2t[r * kS72 + i] = gelu_grad(z, th);
            S.a1[r * kS68 + i] = a;
            S.a1t[r * kS72 + i] = a;
          }
      }
    __syncwarp();
    // ---- layer 2 on the tensor cores
    float acc[kMT][8][4];
#pragma unroll
    for (int mt = 0; mt < kMT; ++mt)
#pragma unroll
      for (int nt = 0; nt < 8; ++nt)
#pragma unroll
        for (int e = 0; e < 4; ++e) acc[mt][nt][e] = 0.f;
    warp_gemm_rows(acc, S.a1, S.w.w2, row0, g, q);
    __syncwarp();  // the warp's a1 rows are read: they now take the layer-1 derivative
    // ---- GELU, output layer, loss, output deltas, layer-2 deltas (C layout)
    float ysum[kMT][2];
#pragma unroll
    for (int mt = 0; mt < kMT; ++mt) ysum[mt][0] = ysum[mt][1] = 0.f;
#pragma unroll
    for (int mt = 0; mt < kMT; ++mt)
#pragma unroll
      for (int nt = 0; nt < 8; ++nt)
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int j = 8 * nt + 2 * q + (e & 1);
          float th;
          const float z = acc[mt][nt][e] + S.w.b2[j];
          const float a2 = gelu_train(z, th);
          ysum[mt][e >> 1] = fmaf(S.w.w3[j], a2, ysum[mt][e >> 1]);
          acc[mt][nt][e] = a2;  // kept for the output-weight gradient
          const int r = row0 + 16 * mt + g + 8 * (e >> 1);
          S.d2[r * kS68 + j] = gelu_grad(z, th);  // GELU'(z2) until the layer-2 delta replaces it
          S.a1[r * kS68 + j] = S.d2t[r * kS72 + j];
        }
    float dyr[kMT][2];
#pragma unroll
    for (int mt = 0; mt < kMT; ++mt)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        float y = ysum[mt][h];
        y += __shfl_xor_sync(0xffffffffu, y, 1);  // the quad's four column sets, in a fixed order
        y += __shfl_xor_sync(0xffffffffu, y, 2);
        const int r = row0 + 16 * mt + g + 8 * h;
        y += S.w.b3[0];
        const bool valid = S.pair[r] >= 0;
        const float res = valid ? y - S.dy[r] : 0.f;
        dyr[mt][h] = res * scale;
        __syncwarp();
        if (q == 0) {
          S.err[r] = res * res;
          S.dy[r] = res * scale;
        }
      }
    // layer-2 deltas; the warp's output-layer gradients (w3, b2) over its 32 samples: per column,
    // the thread's four rows, then the eight row groups (lanes with the same q) in a fixed order
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int j = 8 * nt + 2 * q + u;
        float sw3 = 0.f, sb2 = 0.f;
#pragma unroll
        for (int mt = 0; mt < kMT; ++mt)
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int r = row0 + 16 * mt + g + 8 * h;
            const float d2 = dyr[mt][h] * S.w.w3[j] * S.d2[r * kS68 + j];
            sw3 = fmaf(dyr[mt][h], acc[mt][nt][2 * h + u], sw3);
            sb2 += d2;
            S.d2[r * kS68 + j] = d2;
            S.d2t[r * kS72 + j] = d2;
          }
#pragma unroll
        for (int o = 4; o < 32; o <<= 1) {
          sw3 += __shfl_xor_sync(0xffffffffu, sw3, o);
          sb2 += __shfl_xor_sync(0xffffffffu, sb2, o);
        }
        if (g == 0) {
          S.w_w3[w][j] += sw3;
          S.w_b2[w][j] += sb2;
        }
      }
    __syncwarp();
    // ---- gradient of the layer-1 outputs on the tensor cores: G1 = D2 W2
#pragma unroll
    for (int mt = 0; mt < kMT; ++mt)
#pragma unroll
      for (int nt = 0; nt < 8; ++nt)
#pragma unroll
        for (int e = 0; e < 4; ++e) acc[mt][nt][e] = 0.f;
    warp_gemm_rows(acc, S.d2, S.w.w2t, row0, g, q);
    // layer-1 deltas; the warp's layer-1 gradients (w1, b1) as above, and per sample the
    // gradients of the two embedding inputs (the thread's columns, then the quad)
    float xr[kMT][2][4], dxa[kMT][2][2];
#pragma unroll
    for (int mt = 0; mt < kMT; ++mt)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int r = row0 + 16 * mt + g + 8 * h;
#pragma unroll
        for (int k = 0; k < 4; ++k) xr[mt][h][k] = S.x[r][k];
        dxa[mt][h][0] = dxa[mt][h][1] = 0.f;
      }
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int i = 8 * nt + 2 * q + u;
        float v[5] = {0.f, 0.f, 0.f, 0.f, 0.f};  // b1, w1[i][0..3]
#pragma unroll
        for (int mt = 0; mt < kMT; ++mt)
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const float d1 = acc[mt][nt][2 * h + u] * S.a1[(row0 + 16 * mt + g + 8 * h) * kS68 + i];
            v[0] += d1;
#pragma unroll
            for (int k = 0; k < 4; ++k) v[1 + k] = fmaf(d1, xr[mt][h][k], v[1 + k]);
            dxa[mt][h][0] = fmaf(S.w.w1[4 * i + 2], d1, dxa[mt][h][0]);
            dxa[mt][h][1] = fmaf(S.w.w1[4 * i + 3], d1, dxa[mt][h][1]);
          }
#pragma unroll
        for (int o = 4; o < 32; o <<= 1)
#pragma unroll
          for (int k = 0; k < 5; ++k) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
        if (g == 0) {
          S.w_b1[w][i] += v[0];
#pragma unroll
          for (int k = 0; k < 4; ++k) S.w_w1[w][4 * i + k] += v[1 + k];
        }
      }
#pragma unroll
    for (int mt = 0; mt < kMT; ++mt)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        float dx2 = dxa[mt][h][0], dx3 = dxa[mt][h][1];
        dx2 += __shfl_xor_sync(0xffffffffu, dx2, 1);
        dx2 += __shfl_xor_sync(0xffffffffu, dx2, 2);
        dx3 += __shfl_xor_sync(0xffffffffu, dx3, 1);
        dx3 += __shfl_xor_sync(0xffffffffu, dx3, 2);
        if (q == 0) {
          const int r = row0 + 16 * mt + g + 8 * h;
          S.dx[r][0] = dx2;
          S.dx[r][1] = dx3;
        }
      }
    __syncwarp();
    if (lane == 0) {
      float b3 = 0.f;
      for (int r = row0; r < row0 + 16 * kMT; ++r) b3 += S.dy[r];
      S.w_b3[w] += b3;
    }
    __syncthreads();
    // ---- dW2 += D2^T A1 over the chunk's 128 samples: the warp's 16 x 32 tile
#pragma unroll 1
    for (int ks = 0; ks < kMlpChunk / 8; ++ks) {
      const float* ar = S.d2t + (8 * ks + q) * kS72 + 16 * jt + g;
      uint32_t ah0, al0, ah1, al1, ah2, al2, ah3, al3;
      split_tf32(ar[0], ah0, al0);
      split_tf32(ar[8], ah1, al1);
      split_tf32(ar[4 * kS72], ah2, al2);
      split_tf32(ar[4 * kS72 + 8], ah3, al3);
#pragma unroll
      for (int nt = 0; nt < 4; ++nt) {
        const float* br = S.a1t + (8 * ks + q) * kS72 + 8 * (nt0 + nt) + g;
        uint32_t bh0, bl0, bh1, bl1;
        split_tf32(br[0], bh0, bl0);
        split_tf32(br[4 * kS72], bh1, bl1);
        mma_tf32(acc3[nt], ah0, ah1, ah2, ah3, bh0, bh1);
        mma_tf32(acc3[nt], ah0, ah1, ah2, ah3, bl0, bl1);
        mma_tf32(acc3[nt], al0, al1, al2, al3, bh0, bh1);
      }
    }
    // embedding gradients (entry t & 127: pair / 2, input 2 + entry % 2) over the samples of half
    // t >> 7, in sample order; the loss by warp 0 (four samples a lane, then the lanes) in double
    {
      const int e = t & (kMlpChunk - 1), s0 = (t >> 7) * (kMlpChunk / 2);
      if (e < n_emb)
        for (int s = s0; s < s0 + kMlpChunk / 2; ++s)
          if (S.pair[s] == (e >> 1)) acc_e += S.dx[s][e & 1];
    }
    if (w == 0) {
      double l = 0.0;
      for (int s = lane; s < kMlpChunk; s += 32) l += (double)S.err[s];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
      if (lane == 0) acc_loss += l;
    }
    __syncthreads();
  }
  float* p = part + (int64_t)blockIdx.x * m.n_params;
#pragma unroll
  for (int nt = 0; nt < 4; ++nt)
#pragma unroll
    for (int e = 0; e < 4; ++e)
      p[kMlpOffW2 + (16 * jt + g + 8 * (e >> 1)) * kMlpH + 8 * (nt0 + nt) + 2 * q + (e & 1)] = acc3[nt][e];
  S.emb[t >> 7][t & (kMlpChunk - 1)] = acc_e;
  __syncthreads();
  for (int i = t; i < kMlpH * 4; i += kGradThreads) {
    float v = 0.f;
    for (int k = 0; k < kGradWarps; ++k) v += S.w_w1[k][i];
    p[kMlpOffW1 + i] = v;
  }
  for (int i = t; i < kMlpH; i += kGradThreads) {
    float v1 = 0.f, v2 = 0.f, v3 = 0.f;
    for (int k = 0; k < kGradWarps; ++k) {
      v1 += S.w_b1[k][i];
      v2 += S.w_b2[k][i];
      v3 += S.w_w3[k][i];
    }
    p[kMlpOffB1 + i] = v1;
    p[kMlpOffB2 + i] = v2;
    p[kMlpOffW3 + i] = v3;
  }
  if (t == 0) {
    float v = 0.f;
    for (int k = 0; k < kGradWarps; ++k) v += S.w_b3[k];
    p[kMlpOffB3] = v;
    part_loss[blockIdx.x] = acc_loss;
  }
  if (t < n_emb) p[kMlpOffE + t] = S.emb[0][t] + S.emb[1][t];
}

// Parameter p of the image: matrices from the BF16 copy (bf), the rest from the FP32 master (v).
__device__ __forceinline__ void image_put(const MlpDev& m, int p, float v, uint16_t bf) {
  WeightImage& I = *reinterpret_cast<WeightImage*>(m.image);
  if (p < kMlpOffB1) {
    I.w1[p] = widen(bf);
  } else if (p < kMlpOffW2) {
    I.b1[p - kMlpOffB1] = v;
  } else if (p < kMlpOffB2) {
    const int j = (p - kMlpOffW2) / kMlpH, k = (p - kMlpOffW2) % kMlpH;
    I.w2[j * kS68 + k] = widen(bf);
    I.w2t[k * kS68 + j] = widen(bf);
  } else if (p < kMlpOffW3) {
    I.b2[p - kMlpOffB2] = v;
  } else if (p < kMlpOffB3) {
    I.w3[p - kMlpOffW3] = widen(bf);
  } else if (p < kMlpOffE) {
    if (p == kMlpOffB3) I.b3[0] = v;
  } else {
    I.e[p - kMlpOffE] = v;
  }
}

__global__ void k_mlp_image(MlpDev m) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < m.n_params) image_put(m, p, m.master[p], m.wbf[p]);
}

// The gradient of 32 parameters per block: warp w adds the partials of blocks w, w + 8, ... (lane
// = parameter, coalesced rows), then lane p of warp 0 adds the eight warp sums in warp order, so
// the sum has a fixed order whatever the timing (training stays deterministic) and eight rows of
// partials are in flight at once.  With st.update, one bias-corrected Adam step of the FP32
// master value and its BF16 copy.
constexpr int kUpdWarps = 8;
__global__ void __launch_bounds__(32 * kUpdWarps) k_mlp_update(MlpDev m, float* master, uint16_t* wbf, float* mom1,
                                                               float* mom2, const float* part, const double* part_loss,
                                                               int grid, MlpStep st, float* grad_out, double* loss_out,
                                                               const MlpStep* sched, const unsigned long long* step_ctr) {
  __shared__ float s_sum[kUpdWarps][32];
  if (sched) {
    st = sched[*step_ctr - 1];
    loss_out = st.loss_slot >= 0 ? loss_out + st.loss_slot : nullptr;
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int p = blockIdx.x * 32 + lane;
  if (blockIdx.x == 0 && threadIdx.x == 0 && loss_out) {
    double l = 0.0;
    for (int b = 0; b < grid; ++b) l += part_loss[b];
    *loss_out = l * st.inv_count;
  }
  float g = 0.f;
  if (p < m.n_params) {
    // rows w, w + 8, ... loaded 20 at a time (all in flight), then added in row order
    for (int b0 = w; b0 < grid; b0 += 20 * kUpdWarps) {
      float v[20];
#pragma unroll
      for (int i = 0; i < 20; ++i) {
        const int b = b0 + kUpdWarps * i;
        v[i] = b < grid ? part[(int64_t)b * m.n_params + p] : 0.f;
      }
#pragma unroll
      for (int i = 0; i < 20; ++i) g += v[i];
    }
  }
  s_sum[w][lane] = g;
  __syncthreads();
  if (w != 0 || p >= m.n_params) return;
  g = 0.f;
#pragma unroll
  for (int k = 0; k < kUpdWarps; ++k) g += s_sum[k][lane];
  if (grad_out) grad_out[p] = g;
  if (!st.update) return;
  const float m1 = st.beta1 * mom1[p] + (1.f - st.beta1) * g;
  const float m2 = st.beta2 * mom2[p] + (1.f - st.beta2) * (g * g);
  mom1[p] = m1;
  mom2[p] = m2;
  const float v = master[p] - st.lr * (m1 * st.c1) / (sqrtf(m2 * st.c2) + st.eps);
  master[p] = v;
  const uint16_t bf = __bfloat16_as_ushort(__float2bfloat16_rn(v));
  wbf[p] = bf;
  image_put(m, p, v, bf);
}

__global__ void __launch_bounds__(128) k_mlp_predict(MlpDev m, const double* dist, const double* theta,
                                                      const int32_t* pair, int64_t n, double* out) {
  __shared__ MlpSmem w;
  stage(m, w);
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float y = forward(w, dist_input(m, dist[i]), angle_input(theta[i]), pair[i]);
  out[i] = (double)y * m.log_scale + m.log_mean;
}

// rate[pair][id][it] = exp(ln rate) at (dist[id], theta[it]); pair = donor * S + acceptor
__global__ void __launch_bounds__(128) k_mlp_table(MlpDev m, const double* dist, int32_t nd, const double* theta,
                                                    int32_t nt, double* rate) {
  __shared__ MlpSmem w;
  stage(m, w);
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t per_pair = (int64_t)nd * nt;
  if (i >= per_pair * m.n_species * m.n_species) return;
  const int pair = (int)(i / per_pair);
  const int64_t r = i - pair * per_pair;
  const int id = (int)(r / nt), it = (int)(r - (int64_t)id * nt);
  const float y = forward(w, dist_input(m, dist[id]), angle_input(theta[it]), pair);
  rate[i] = exp((double)y * m.log_scale + m.log_mean);
}

}  // namespace

size_t mlp_grad_smem_bytes() { return sizeof(GradSmem); }

cudaError_t launch_mlp_samples(const MlpDev& m, const double* dist, const double* theta, const int32_t* pair,
                               const double* log_rate, int64_t n, float4* out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_mlp_samples<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(m, dist, theta, pair, log_rate, n, out);
  return cudaGetLastError();
}

cudaError_t launch_mlp_bf16(const float* master, uint16_t* wbf, int32_t n, cudaStream_t s) {
  k_mlp_bf16<<<(n + 255) / 256, 256, 0, s>>>(master, wbf, n);
  return cudaGetLastError();
}

cudaError_t launch_mlp_grad(const MlpDev& m, const float4* samples, int64_t first, int64_t count, float* part,
                            double* part_loss, int grid, cudaStream_t s, unsigned long long* step_ctr) {
  const size_t bytes = mlp_grad_smem_bytes();
  static thread_local int opted = -1;  // the shared-memory opt-in, once per thread and device
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (opted != dev) {
    e = cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) return e;
    opted = dev;
  }
  k_mlp_grad<<<grid, kGradThreads, bytes, s>>>(m, samples, first, count, part, part_loss, step_ctr);
  return cudaGetLastError();
}

cudaError_t launch_mlp_image(const MlpDev& m, cudaStream_t s) {
  k_mlp_image<<<(m.n_params + 255) / 256, 256, 0, s>>>(m);
  return cudaGetLastError();
}

cudaError_t launch_mlp_update(const MlpDev& m, float* master, uint16_t* wbf, float* mom1, float* mom2,
                              const float* part, const double* part_loss, int grid, const MlpStep& st,
                              float* grad_out, double* loss_out, cudaStream_t s, const MlpStep* sched,
                              const unsigned long long* step_ctr) {
  k_mlp_update<<<(m.n_params + 31) / 32, 32 * kUpdWarps, 0, s>>>(m, master, wbf, mom1, mom2, part, part_loss,
                                                                         grid, st, grad_out, loss_out, sched, step_ctr);
  return cudaGetLastError();
}

cudaError_t launch_mlp_predict(const MlpDev& m, const double* dist, const double* theta, const int32_t* pair,
                               int64_t n, double* log_rate, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_mlp_predict<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(m, dist, theta, pair, n, log_rate);
  return cudaGetLastError();
}

cudaError_t launch_mlp_table(const MlpDev& m, const double* dist, int32_t nd, const double* theta, int32_t nt,
                             double* rate, cudaStream_t s) {
  const int64_t n = (int64_t)nd * nt * m.n_species * m.n_species;
  if (n <= 0) return cudaSuccess;
  k_mlp_table<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(m, dist, nd, theta, nt, rate);
  return cudaGetLastError();
}

}  // namespace kmc
