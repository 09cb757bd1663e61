// Plain FP32 MLP building blocks for the DIVeR decoder (per-thread rows).
//
// Weights live in shared memory in the packed torch layout: each Linear layer
// as W^T [in][out4] row-major (out4 = out rounded up to 4) followed by its
// bias [out4].  A thread evaluates one segment: activations are register
// arrays, every weight row is read as float4 broadcasts (all threads of a
// warp read the same address).
#pragma once
#include <cuda_runtime.h>

namespace dv {

constexpr int PE_DIM = 27;   // 3 + 3*2*4 (model/mlps.py:6-18, L = 4)
constexpr int PE_PAD = 28;

__host__ __device__ constexpr int pad4(int n) { return (n + 3) & ~3; }

// y[0:OUT4) = b + x[0:IN) @ Wt (x optionally through ReLU first).
template <int IN, int OUT4, bool RELU_IN, bool BIAS = true>
__device__ __forceinline__ void dense_fwd(const float* __restrict__ Wt, const float* __restrict__ b,
                                          const float* x, float* y) {
#pragma unroll
  for (int j = 0; j < OUT4; j += 4) {
    if (BIAS) {
      const float4 v = *reinterpret_cast<const float4*>(b + j);
      y[j] = v.x;
      y[j + 1] = v.y;
      y[j + 2] = v.z;
      y[j + 3] = v.w;
    } else {
      y[j] = y[j + 1] = y[j + 2] = y[j + 3] = 0.f;
    }
  }
#pragma unroll
  for (int i = 0; i < IN; ++i) {
    const float xi = RELU_IN ? fmaxf(x[i], 0.f) : x[i];
#pragma unroll
    for (int j = 0; j < OUT4; j += 4) {
      const float4 w = *reinterpret_cast<const float4*>(Wt + i * OUT4 + j);
      y[j] = fmaf(xi, w.x, y[j]);
      y[j + 1] = fmaf(xi, w.y, y[j + 1]);
      y[j + 2] = fmaf(xi, w.z, y[j + 2]);
      y[j + 3] = fmaf(xi, w.w, y[j + 3]);
    }
  }
}

// y[0:OUT4) = b + xs[0:in) @ Wt with xs the thread's own shared-memory row
// (optionally through ReLU): only the output dimension is unrolled, which
// keeps wide layers small to compile.
template <int OUT4, bool RELU_IN, bool BIAS = true>
__device__ __forceinline__ void dense_fwd_s(const float* __restrict__ Wt, const float* __restrict__ b,
                                            const float* xs, int in, float* y) {
#pragma unroll
  for (int j = 0; j < OUT4; j += 4) {
    if (BIAS) {
      const float4 v = *reinterpret_cast<const float4*>(b + j);
      y[j] = v.x;
      y[j + 1] = v.y;
      y[j + 2] = v.z;
      y[j + 3] = v.w;
    } else {
      y[j] = y[j + 1] = y[j + 2] = y[j + 3] = 0.f;
    }
  }
#pragma unroll 2
  for (int i = 0; i < in; ++i) {
    const float xi = RELU_IN ? fmaxf(xs[i], 0.f) : xs[i];
    const float* row = Wt + i * OUT4;
#pragma unroll
    for (int j = 0; j < OUT4; j += 4) {
      const float4 w = *reinterpret_cast<const float4*>(row + j);
      y[j] = fmaf(xi, w.x, y[j]);
      y[j + 1] = fmaf(xi, w.y, y[j + 1]);
      y[j + 2] = fmaf(xi, w.z, y[j + 2]);
      y[j + 3] = fmaf(xi, w.w, y[j + 3]);
    }
  }
}

// dxs[i] = mask(i) * (Wt[i] . d) for i < in, into the thread's own shared row;
// mask(i) = (act[i] > 0) when act is given (ReLU derivative), else 1.
template <int OUT4>
__device__ __forceinline__ void dense_bwd_input_s(const float* __restrict__ Wt, const float* d, int in, const float* act,
                                                  float* dxs) {
#pragma unroll 2
  for (int i = 0; i < in; ++i) {
    const float* row = Wt + i * OUT4;
    float acc = 0.f;
#pragma unroll
    for (int j = 0; j < OUT4; j += 4) {
      const float4 w = *reinterpret_cast<const float4*>(row + j);
      acc = fmaf(w.x, d[j], acc);
      acc = fmaf(w.y, d[j + 1], acc);
      acc = fmaf(w.z, d[j + 2], acc);
      acc = fmaf(w.w, d[j + 3], acc);
    }
    dxs[i] = (act == nullptr || act[i] > 0.f) ? acc : 0.f;
  }
}

// dx[0:IN) = Wt[0:IN) @ d  (d has OUT4 entries, zero past the layer's out).
template <int IN, int OUT4>
__device__ __forceinline__ void dense_bwd_input(const float* __restrict__ Wt, const float* d, float* dx) {
#pragma unroll
  for (int i = 0; i < IN; ++i) {
    float acc = 0.f;
#pragma unroll
    for (int j = 0; j < OUT4; j += 4) {
      const float4 w = *reinterpret_cast<const float4*>(Wt + i * OUT4 + j);
      acc = fmaf(w.x, d[j], acc);
      acc = fmaf(w.y, d[j + 1], acc);
      acc = fmaf(w.z, d[j + 2], acc);
      acc = fmaf(w.w, d[j + 3], acc);
    }
    dx[i] = acc;
  }
}

__device__ __forceinline__ float sigmoidf_acc(float x) { return 1.f / (1.f + expf(-x)); }

// Positional encoding of a direction, reference order
// [d, sin(pi d), cos(pi d), sin(2pi d), cos(2pi d), ..., cos(8pi d)] with
// 3-vectors per entry (model/mlps.py:10-18); pe[27] = 0.
__device__ __forceinline__ void pos_enc(float dx, float dy, float dz, float* pe) {
  pe[0] = dx;
  pe[1] = dy;
  pe[2] = dz;
  float f = 3.14159265358979323846f;
#pragma unroll
  for (int l = 0; l < 4; ++l) {
    float s, c;
    sincosf(f * dx, &s, &c);
    pe[3 + 6 * l + 0] = s;
    pe[3 + 6 * l + 3] = c;
    sincosf(f * dy, &s, &c);
    pe[3 + 6 * l + 1] = s;
    pe[3 + 6 * l + 4] = c;
    sincosf(f * dz, &s, &c);
    pe[3 + 6 * l + 2] = s;
    pe[3 + 6 * l + 5] = c;
    f *= 2.f;
  }
  pe[27] = 0.f;
}

}  // namespace dv
