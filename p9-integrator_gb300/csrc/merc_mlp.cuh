// merc_mlp.cuh - learned warm start of the universal-variable Kepler solve.
//
// A 4 -> 32 -> 32 -> 1 SiLU network in FP32 predicts the universal anomaly s
// of a drift.  With mu = 1, r0 = |x0|, eta = x0.v0, alpha = 2/r0 - v0^2, the
// plain guess is s0 = dt / r0, and the drift is fixed by the dimensionless
//   x1 = dt / r0^1.5,  x2 = r0 v0^2,  x3 = eta / sqrt(r0),  x4 = sign of the energy.
// The solution is written s = s0 exp(z) with
//   z = -x1 x3 / (2 (1 + x1^2)) + y x1^2 / (1 + x1^2):
// for short drifts (x1 << 1) z tends to its series -x1 x3 / 2 + O(x1^2) and
// the network's error in y enters scaled by x1^2; for long ones (pericentre
// passages, hyperbolic flybys, x1 up to ~10) s/s0 ranges over a factor ~30
// and the error in y enters unscaled.  The network sees ln x1, x2, x3, x4
// (the logged samples store ln x1), normalised by the training set's mean and
// spread, and predicts y.  At inference the features and exp(z) - 1 are
// computed in FP32 (warm_features_f32, warm_delta) and the drift forms
// s0 (1 + delta) from its own FP64 s0.  The FP64 Newton solve that follows is
// unchanged; the guess only moves its starting point.  Outside the feature box
// seen in training, and for short drifts (x1 < kWarmNetX1, where the series
// guess needs one iteration), the series guess is used.
//
// Parameter blob (floats): W1[32][4], b1[32], W2[32][32], b2[32], W3[32], b3,
// then in_mean[4], in_scale[4], out_mean, out_scale, box_lo[4], box_hi[4].
#pragma once

namespace {

constexpr int kH = 32;
constexpr int kNet = kH * 4 + kH + kH * kH + kH + kH + 1;  // 1249
constexpr int kBlob = kNet + 18;
constexpr int kW1 = 0, kB1 = kW1 + kH * 4, kW2 = kB1 + kH, kB2 = kW2 + kH * kH, kW3 = kB2 + kH, kB3 = kW3 + kH;
constexpr int kInMean = kNet, kInScale = kNet + 4, kOutMean = kNet + 8, kOutScale = kNet + 9, kBoxLo = kNet + 10,
              kBoxHi = kNet + 14;

struct WarmIn {
  float f[4];   // raw features x1..x4
  double s0;    // plain guess dt / r0
};

__device__ __forceinline__ WarmIn warm_features(const d3& x0, const d3& v0, double dt) {
  double r0 = sqrt(mag2(x0));
  double eta = fma(x0.x, v0.x, fma(x0.y, v0.y, x0.z * v0.z));
  double v2 = mag2(v0);
  double sr = sqrt(r0);
  WarmIn w;
  w.s0 = dt / r0;
  w.f[0] = (float)(dt / (r0 * sr));
  w.f[1] = (float)(r0 * v2);
  w.f[2] = (float)(eta / sr);
  w.f[3] = (2.0 - r0 * v2) < 0.0 ? 1.0f : -1.0f;  // alpha r0 = 2 - r0 v0^2; energy > 0 iff alpha < 0
  return w;
}

// The same features in FP32 from the high-word truncations of x0, v0 and dt
// (each within 2^-20): no FP64 square root, division or conversion.  The
// guess they feed needs ~1e-6; the FP64 Newton solve that follows is
// unchanged.
__device__ __forceinline__ void warm_features_f32(const d3& x0, const d3& v0, float dtf, float f[4]) {
  const float x = f32_trunc(x0.x), y = f32_trunc(x0.y), z = f32_trunc(x0.z);
  const float vx = f32_trunc(v0.x), vy = f32_trunc(v0.y), vz = f32_trunc(v0.z);
  const float r2 = fmaf(x, x, fmaf(y, y, z * z));
  const float ir = rsqrtf(r2), r0 = r2 * ir, isr = sqrtf(ir);  // 1/r0, r0, 1/sqrt(r0)
  const float v2 = fmaf(vx, vx, fmaf(vy, vy, vz * vz)), eta = fmaf(x, vx, fmaf(y, vy, z * vz));
  f[0] = dtf * ir * isr;
  f[1] = r0 * v2;
  f[2] = eta * isr;
  f[3] = (2.0f - r0 * v2) < 0.0f ? 1.0f : -1.0f;
}

// The network is consulted only for drifts with x1 >= kWarmNetX1: below it the
// series guess already converges in one Newton iteration (the embryo disk,
// x1 ~ 0.01, the sweep and the planetesimal disk) and the network's ~1200 FP32
// multiply-adds per body would cost more than they save.  warm_long decides
// it from FP32 truncations without a root: x1^4 = dt^4 / r0^6 >= kWarmNetX1^4.
constexpr float kWarmNetX1 = 0.03f;
__device__ __forceinline__ bool warm_long(const d3& x0, float dtf) {
  const float x = f32_trunc(x0.x), y = f32_trunc(x0.y), z = f32_trunc(x0.z);
  const float r2 = fmaf(x, x, fmaf(y, y, z * z));
  const float d2 = dtf * dtf, g2 = kWarmNetX1 * kWarmNetX1;
  return d2 * d2 >= (g2 * g2) * (r2 * r2 * r2);
}

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }

// forward pass on normalised inputs; p points at the blob (shared or global)
__device__ __forceinline__ float mlp_forward(const float* __restrict__ p, const float* xn) {
  float h1[kH];
#pragma unroll
  for (int i = 0; i < kH; i++) {
    float z = p[kB1 + i];
#pragma unroll
    for (int k = 0; k < 4; k++) z = fmaf(p[kW1 + 4 * i + k], xn[k], z);
    h1[i] = silu(z);
  }
  float y = p[kB3];
#pragma unroll 4
  for (int i = 0; i < kH; i++) {
    float z = p[kB2 + i];
#pragma unroll
    for (int k = 0; k < kH; k++) z = fmaf(p[kW2 + kH * i + k], h1[k], z);
    y = fmaf(p[kW3 + i], silu(z), y);
  }
  return y;
}

// Relative correction of the plain guess, s = (dt / r0) (1 + delta), from
// FP32 features x1..x4; NaN outside the trained feature box.
__device__ __forceinline__ float warm_delta(const float* __restrict__ p, const float f[4]) {
  const float u[4] = {__logf(f[0]), f[1], f[2], f[3]};
  float xn[4];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    if (!(u[k] >= p[kBoxLo + k] && u[k] <= p[kBoxHi + k])) return __int_as_float(0x7fc00000);
    xn[k] = (u[k] - p[kInMean + k]) * p[kInScale + k];
  }
  const float y = mlp_forward(p, xn) / p[kOutScale] + p[kOutMean];
  const float q = f[0] * f[0], iq = 1.0f / (1.0f + q);
  return expm1f(iq * fmaf(y, q, -0.5f * f[0] * f[2]));
}

// logged network input 0 of a drift: ln x1
__device__ __forceinline__ float warm_input0(const WarmIn& w) { return (float)log((double)w.f[0]); }

// training target y of a solved drift: (ln(s/s0) + x1 x3 / (2 (1 + x1^2))) (1 + x1^2) / x1^2
__device__ __forceinline__ float warm_target(const WarmIn& w, double s) {
  const double x1 = (double)w.f[0], x3 = (double)w.f[2], q = x1 * x1;
  return (float)((log(s / w.s0) + 0.5 * x1 * x3 / (1.0 + q)) * (1.0 + q) / q);
}

// ---------------------------------------------------------------------------
// training: per-sample forward/backward in registers, gradients summed over
// the warp by shuffles, over the block in shared memory, and written as one
// partial per block; k_mlp_reduce adds the block partials in block order
// (deterministic) and k_mlp_adam applies Adam.
// ---------------------------------------------------------------------------
constexpr int kMlpThreads = 128;

// Loss 0.5 (f(xn) - t)^2 per sample.  Samples come from `data` (5 floats per
// sample: ln x1, x2, x3, x4, target y), drawn by index hash from [0, n_data);
// normalisation from the blob.  grad_part: [gridDim.x][kNet + 1] (last = loss).
__global__ void __launch_bounds__(kMlpThreads) k_mlp_grad(const float* __restrict__ blob,
                                                          const float* __restrict__ data, long long n_data,
                                                          const long long* __restrict__ index, int batch,
                                                          unsigned long long seed, float* __restrict__ grad_part) {
  __shared__ float p[kBlob];
  __shared__ float acc[kNet + 1];
  for (int k = threadIdx.x; k < kBlob; k += blockDim.x) p[k] = blob[k];
  for (int k = threadIdx.x; k < kNet + 1; k += blockDim.x) acc[k] = 0.0f;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  for (int b0 = blockIdx.x * blockDim.x; b0 < batch; b0 += gridDim.x * blockDim.x) {
    const int b = b0 + threadIdx.x;
    const bool act = b < batch;
    long long idx = 0;
    if (act) {
      if (index) {
        idx = index[b];
      } else {  // splitmix64 of (seed, b)
        unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(b + 1);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        idx = (long long)(z % (unsigned long long)n_data);
      }
    }
    float xn[4], t = 0.0f;
    for (int k = 0; k < 4; k++) xn[k] = act ? (data[5 * idx + k] - p[kInMean + k]) * p[kInScale + k] : 0.0f;
    t = act ? (data[5 * idx + 4] - p[kOutMean]) * p[kOutScale] : 0.0f;
    // forward, keeping pre-activations
    float z1[kH], h1[kH], z2[kH], h2[kH];
    for (int i = 0; i < kH; i++) {
      float z = p[kB1 + i];
      for (int k = 0; k < 4; k++) z = fmaf(p[kW1 + 4 * i + k], xn[k], z);
      z1[i] = z;
      h1[i] = silu(z);
    }
    float y = p[kB3];
    for (int i = 0; i < kH; i++) {
      float z = p[kB2 + i];
      for (int k = 0; k < kH; k++) z = fmaf(p[kW2 + kH * i + k], h1[k], z);
      z2[i] = z;
      h2[i] = silu(z);
      y = fmaf(p[kW3 + i], h2[i], y);
    }
    const float e = act ? (y - t) : 0.0f;  // dL/dy
    // backward; silu'(z) = s (1 + z (1 - s)), s = sigmoid(z)
    float d2[kH], d1[kH];
    for (int i = 0; i < kH; i++) {
      float s = 1.0f / (1.0f + __expf(-z2[i]));
      d2[i] = e * p[kW3 + i] * (s * (1.0f + z2[i] * (1.0f - s)));
    }
    for (int k = 0; k < kH; k++) {
      float g = 0.0f;
      for (int i = 0; i < kH; i++) g = fmaf(p[kW2 + kH * i + k], d2[i], g);
      float s = 1.0f / (1.0f + __expf(-z1[k]));
      d1[k] = g * (s * (1.0f + z1[k] * (1.0f - s)));
    }
    // gradients, summed over the warp then added to the block accumulator
    auto put = [&](int slot, float v) {
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) atomicAdd(&acc[slot], v);
    };
    for (int i = 0; i < kH; i++) {
      for (int k = 0; k < 4; k++) put(kW1 + 4 * i + k, d1[i] * xn[k]);
      put(kB1 + i, d1[i]);
    }
    for (int i = 0; i < kH; i++) {
      for (int k = 0; k < kH; k++) put(kW2 + kH * i + k, d2[i] * h1[k]);
      put(kB2 + i, d2[i]);
      put(kW3 + i, e * h2[i]);
    }
    put(kB3, e);
    put(kNet, 0.5f * e * e);
  }
  __syncthreads();
  for (int k = threadIdx.x; k < kNet + 1; k += blockDim.x) grad_part[(size_t)blockIdx.x * (kNet + 1) + k] = acc[k];
}

// sum of the block partials in block order, divided by the batch
__global__ void k_mlp_reduce(const float* __restrict__ grad_part, int nblocks, int batch, float* __restrict__ grad) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k > kNet) return;
  float s = 0.0f;
  for (int b = 0; b < nblocks; b++) s += grad_part[(size_t)b * (kNet + 1) + k];
  grad[k] = s / (float)batch;
}

__global__ void k_mlp_adam(float* __restrict__ blob, const float* __restrict__ grad, float* __restrict__ m,
                           float* __restrict__ v, float lr, float b1, float b2, float eps, int step) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= kNet) return;
  float g = grad[k];
  float mk = b1 * m[k] + (1.0f - b1) * g;
  float vk = b2 * v[k] + (1.0f - b2) * g * g;
  m[k] = mk;
  v[k] = vk;
  float mh = mk / (1.0f - powf(b1, (float)step));
  float vh = vk / (1.0f - powf(b2, (float)step));
  blob[k] -= lr * mh / (sqrtf(vh) + eps);
}

}  // namespace
