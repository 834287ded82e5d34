// kmc_mlp.cu -- the learned pair-rate surrogate: training (forward + backward + Adam), inference
// and the table builder that turns the network into a KMC_TABLE_2D_SPECIES rate table.
//
// The network is tiny (4 -> 64 -> 64 -> 1, 4.6k parameters) and a 2M-sample epoch is ~55 GFLOP,
// so one thread carries one sample through the whole network with the weights staged in shared
// memory (every lane reads the same weight at the same time: broadcasts), and the weight
// gradients are reduced per block over its samples in a fixed order (outer products read from
// shared memory), then across blocks in block order: training is deterministic.
#include <cuda_bf16.h>

#include "../../include/cntkmc.h"
#include "kmc_internal.h"

namespace kmc {
namespace {

constexpr float kGeluK0 = 0.7978845608028654f;  // sqrt(2 / pi), GELU tanh form (Hendrycks & Gimpel)
constexpr float kGeluK1 = 0.044715f;
constexpr double kThetaScale = 1.2732395447351628;  // 4 / pi: theta in [0, pi/2] -> [0, 2]
constexpr int kAcc = kMlpH / 2 + 5;  // gradient sums per thread in the gradient kernel
constexpr int kRow = kMlpH + 1;  // activation rows padded to 65 words: thread s writing word i of
                                 // its row hits bank (s + i) mod 32

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

// Gradient of sum_k (y_k - label_k)^2 / count over samples [first, first + count).  Block b takes
// chunks b, b + grid, ... of 128 samples, one per thread: forward and backward of its sample,
// activations and deltas into shared rows, then the block's weight gradients as sums over the
// chunk's samples in sample order.  Thread t owns W2 row t/2, columns 2q + (t & 1) (adjacent
// lanes read adjacent words), W1 row t/2, columns 2 (t & 1) .. +1, b1[t] or b2[t - 64], W3[t] or
// b3 (t = 64), and embedding entry t.  Each block writes its partials to part[b][*].
__global__ void __launch_bounds__(kMlpChunk, 1)
    k_mlp_grad(MlpDev m, const float4* smp, int64_t first, int64_t count, float* part, double* part_loss) {
  extern __shared__ __align__(16) unsigned char smem[];
  MlpSmem& w = *reinterpret_cast<MlpSmem*>(smem);
  float* s_a1 = reinterpret_cast<float*>(smem + sizeof(MlpSmem));  // [128][65] layer-1 outputs
  float* s_a2 = s_a1 + kMlpChunk * kRow;                            // [128][65] layer-2 outputs
  float* s_d2 = s_a2 + kMlpChunk * kRow;                            // [128][65] GELU'(z2), then layer-2 deltas
  float* s_d1 = s_d2 + kMlpChunk * kRow;                            // [128][65] GELU'(z1), then layer-1 deltas
  float* s_x = s_d1 + kMlpChunk * kRow;                             // [128][5] inputs
  float* s_dx = s_x + kMlpChunk * 5;                                // [128][2] embedding gradients
  float* s_dy = s_dx + kMlpChunk * 2;                               // [128] output deltas
  float* s_err = s_dy + kMlpChunk;                                  // [128] squared errors
  int* s_pair = reinterpret_cast<int*>(s_err + kMlpChunk);          // [128] pair, -1 past the end
                                                                    // then [kAcc][128] running sums
  stage(m, w);
  const int t = threadIdx.x;
  const int jr = t >> 1, half = t & 1;
  const int n_emb = 2 * m.n_species * m.n_species;
  const float scale = (float)(2.0 / (double)count);
  // the thread's running sums live in shared memory between chunks (column t of s_acc), so that
  // the forward and backward passes have the registers to themselves
  float* acc = reinterpret_cast<float*>(s_pair + kMlpChunk) + t;  // acc[q * 128], q < kAcc
#pragma unroll
  for (int q = 0; q < kAcc; ++q) acc[q * kMlpChunk] = 0.f;
  double acc_loss = 0.0;
  const int64_t n_chunks = (count + kMlpChunk - 1) / kMlpChunk;
  float* row_a1 = s_a1 + t * kRow;
  float* row_a2 = s_a2 + t * kRow;
  float* row_d2 = s_d2 + t * kRow;
  float* row_d1 = s_d1 + t * kRow;
  for (int64_t c = blockIdx.x; c < n_chunks; c += gridDim.x) {
    const int64_t k = c * kMlpChunk + t;
    const bool valid = k < count;
    const float4 sm = valid ? smp[first + k] : make_float4(0.f, 0.f, 0.f, 0.f);
    const int pair = valid ? __float_as_int(sm.z) : 0;
    const float x0 = sm.x, x1 = sm.y, x2 = w.e[2 * pair], x3 = w.e[2 * pair + 1];
    // forward
    float a[kMlpH];
#pragma unroll
    for (int i = 0; i < kMlpH; ++i) {
      const float z = layer1(w, i, x0, x1, x2, x3);
      float th;
      a[i] = gelu(z, th);
      row_a1[i] = a[i];
      row_d1[i] = gelu_grad(z, th);
    }
    float y = w.b3[0];
#pragma unroll 1
    for (int j = 0; j < kMlpH; ++j) {
      const float z = row_dot(w, j, a);
      float th;
      const float a2 = gelu(z, th);
      row_a2[j] = a2;
      row_d2[j] = gelu_grad(z, th);
      y = fmaf(w.w3[j], a2, y);
    }
    const float r = valid ? y - sm.w : 0.f;
    const float dy = r * scale;
    // backward through layer 2: a[] becomes the gradient of the layer-1 outputs
#pragma unroll
    for (int i = 0; i < kMlpH; ++i) a[i] = 0.f;
#pragma unroll 1
    for (int j = 0; j < kMlpH; ++j) {
      const float d2 = dy * w.w3[j] * row_d2[j];
      row_d2[j] = d2;
      const float4* rw = reinterpret_cast<const float4*>(w.w2 + j * kMlpH);
#pragma unroll
      for (int q = 0; q < kMlpH / 4; ++q) {
        const float4 cw = rw[q];
        a[4 * q] = fmaf(cw.x, d2, a[4 * q]);
        a[4 * q + 1] = fmaf(cw.y, d2, a[4 * q + 1]);
        a[4 * q + 2] = fmaf(cw.z, d2, a[4 * q + 2]);
        a[4 * q + 3] = fmaf(cw.w, d2, a[4 * q + 3]);
      }
    }
    // layer 1 and the embedding inputs
    float dx2 = 0.f, dx3 = 0.f;
#pragma unroll
    for (int i = 0; i < kMlpH; ++i) {
      const float d1 = a[i] * row_d1[i];
      row_d1[i] = d1;
      dx2 = fmaf(w.w1[4 * i + 2], d1, dx2);
      dx3 = fmaf(w.w1[4 * i + 3], d1, dx3);
    }
    s_x[t * 5] = x0;
    s_x[t * 5 + 1] = x1;
    s_x[t * 5 + 2] = x2;
    s_x[t * 5 + 3] = x3;
    s_dx[2 * t] = dx2;
    s_dx[2 * t + 1] = dx3;
    s_dy[t] = dy;
    s_err[t] = r * r;
    s_pair[t] = valid ? pair : -1;
    __syncthreads();
    // the block's sums over the chunk, in sample order
    float acc_w2[kMlpH / 2];
#pragma unroll
    for (int q = 0; q < kMlpH / 2; ++q) acc_w2[q] = acc[q * kMlpChunk];
    float acc_w1a = acc[32 * kMlpChunk], acc_w1b = acc[33 * kMlpChunk], acc_b = acc[34 * kMlpChunk];
    float acc_w3 = acc[35 * kMlpChunk], acc_e = acc[36 * kMlpChunk];
    for (int s = 0; s < kMlpChunk; ++s) {
      const float* a1s = s_a1 + s * kRow;
      const float d2j = s_d2[s * kRow + jr];
#pragma unroll
      for (int q = 0; q < kMlpH / 2; ++q) acc_w2[q] = fmaf(d2j, a1s[2 * q + half], acc_w2[q]);
      const float d1j = s_d1[s * kRow + jr];
      acc_w1a = fmaf(d1j, s_x[s * 5 + 2 * half], acc_w1a);
      acc_w1b = fmaf(d1j, s_x[s * 5 + 2 * half + 1], acc_w1b);
      if (t < kMlpH) {
        acc_b += s_d1[s * kRow + t];
        acc_w3 = fmaf(s_dy[s], s_a2[s * kRow + t], acc_w3);
      } else {
        acc_b += s_d2[s * kRow + t - kMlpH];
        if (t == kMlpH) acc_w3 += s_dy[s];
      }
      if (t < n_emb && s_pair[s] == (t >> 1)) acc_e += s_dx[2 * s + (t & 1)];
      if (t == 0) acc_loss += (double)s_err[s];
    }
#pragma unroll
    for (int q = 0; q < kMlpH / 2; ++q) acc[q * kMlpChunk] = acc_w2[q];
    acc[32 * kMlpChunk] = acc_w1a;
    acc[33 * kMlpChunk] = acc_w1b;
    acc[34 * kMlpChunk] = acc_b;
    acc[35 * kMlpChunk] = acc_w3;
    acc[36 * kMlpChunk] = acc_e;
    __syncthreads();
  }
  float acc_w2[kMlpH / 2];
#pragma unroll
  for (int q = 0; q < kMlpH / 2; ++q) acc_w2[q] = acc[q * kMlpChunk];
  const float acc_w1a = acc[32 * kMlpChunk], acc_w1b = acc[33 * kMlpChunk], acc_b = acc[34 * kMlpChunk];
  const float acc_w3 = acc[35 * kMlpChunk], acc_e = acc[36 * kMlpChunk];
  float* p = part + (int64_t)blockIdx.x * m.n_params;
#pragma unroll
  for (int q = 0; q < kMlpH / 2; ++q) p[kMlpOffW2 + jr * kMlpH + 2 * q + half] = acc_w2[q];
  p[kMlpOffW1 + jr * 4 + 2 * half] = acc_w1a;
  p[kMlpOffW1 + jr * 4 + 2 * half + 1] = acc_w1b;
  if (t < kMlpH) {
    p[kMlpOffB1 + t] = acc_b;
    p[kMlpOffW3 + t] = acc_w3;
  } else {
    p[kMlpOffB2 + t - kMlpH] = acc_b;
    if (t == kMlpH) p[kMlpOffB3] = acc_w3;
  }
  if (t < n_emb) p[kMlpOffE + t] = acc_e;
  if (t == 0) part_loss[blockIdx.x] = acc_loss;
}

// Thread p: the gradient of parameter p summed over the blocks' partials in block order; with
// st.update, one bias-corrected Adam step of the FP32 master value and its BF16 copy.
__global__ void k_mlp_update(MlpDev m, float* master, uint16_t* wbf, float* mom1, float* mom2, const float* part,
                             const double* part_loss, int grid, MlpStep st, float* grad_out, double* loss_out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p == 0 && loss_out) {
    double l = 0.0;
    for (int b = 0; b < grid; ++b) l += part_loss[b];
    *loss_out = l * st.inv_count;
  }
  if (p >= m.n_params) return;
  float g = 0.f;
  for (int b = 0; b < grid; ++b) g += part[(int64_t)b * m.n_params + p];
  if (grad_out) grad_out[p] = g;
  if (!st.update) return;
  const float m1 = st.beta1 * mom1[p] + (1.f - st.beta1) * g;
  const float m2 = st.beta2 * mom2[p] + (1.f - st.beta2) * (g * g);
  mom1[p] = m1;
  mom2[p] = m2;
  const float v = master[p] - st.lr * (m1 * st.c1) / (sqrtf(m2 * st.c2) + st.eps);
  master[p] = v;
  wbf[p] = __bfloat16_as_ushort(__float2bfloat16_rn(v));
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

size_t mlp_grad_smem_bytes() {
  return sizeof(MlpSmem) + (size_t)kMlpChunk * (4 * kRow + 5 + 2 + 1 + 1 + 1 + kAcc) * sizeof(float);
}

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
                            double* part_loss, int grid, cudaStream_t s) {
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
  k_mlp_grad<<<grid, kMlpChunk, bytes, s>>>(m, samples, first, count, part, part_loss);
  return cudaGetLastError();
}

cudaError_t launch_mlp_update(const MlpDev& m, float* master, uint16_t* wbf, float* mom1, float* mom2,
                              const float* part, const double* part_loss, int grid, const MlpStep& st,
                              float* grad_out, double* loss_out, cudaStream_t s) {
  k_mlp_update<<<(m.n_params + 255) / 256, 256, 0, s>>>(m, master, wbf, mom1, mom2, part, part_loss, grid, st,
                                                         grad_out, loss_out);
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
