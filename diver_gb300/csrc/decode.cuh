// Segment-parallel decode for the training / offline path, plain FP32
// (kernel templates; each decoder variant is instantiated in its own
// translation unit, decode_v<width>c<channels>.cu).
//
//   decode_fwd_plain  gather + integrate + mlp1 + mlp2 + sigmoid per segment
//   decode_bwd_plain  recompute + backprop through the MLPs and the integral:
//                     feature-grid gradient (vector atomics) and MLP weight
//                     gradient (per-CTA shared-memory accumulation)
//
// Reference semantics: model/diver.py:159-180 (decode), utils/integrator.py:
// 62-112 (integral).  A CTA works on tiles of TILE segments: the integral is
// gathered cooperatively (C/4 threads per segment, coalesced float4 loads of
// each corner row) into a shared-memory feature tile, then one thread runs one
// segment's MLP with its activations in its own shared-memory rows and the
// weights broadcast from shared memory.
#pragma once
#include "common.cuh"
#include "integrate.cuh"
#include "mlp.cuh"

#include <algorithm>

namespace dv {

constexpr int MAX_LAYERS = 5;

struct DecodeArgs {
  const float* grid;
  int nvx, nvy, nvz;
  const float* seg;        // [S][6]
  const int* seg_ray;      // [S]
  long long S;             // segment count, or capacity when S_dev is set
  const int64_t* S_dev;    // optional device-held count (clamped to S)
  const int64_t* offsets;  // [B+1]
  int B;
  const float* params;     // packed plain layout
  int n_params;            // multiple of 4
  int w_off[MAX_LAYERS];
  int b_off[MAX_LAYERS];
  const float* dirs;       // [B][3]
  float* pe_feat;          // [B][28]   PE values
  float* pe_out;           // [B][W]    b + PE @ Wt(pe rows) of mlp2's first layer
  float4* out4;            // [S] (sigma_raw, r, g, b)
  const float4* d4;        // [S] (dL/dsigma_raw, dL/dr, dL/dg, dL/db)
  float* grad_grid;        // accumulated
  float* grad_params;      // accumulated, packed layout
  int white_back;
  float* rgb;              // [B][3]
  float* t_final;          // [B] or null
  float* reg_sum;          // [B] or null: sum of log(1 + sigma^2 / 0.5)
  const float* g_rgb;      // [B][3] dL/drgb
  float reg_coef;          // l_s / (B * M), or l_s / B with reg_scale = 1 / M
  const float* reg_scale;  // optional device factor on reg_coef
  float* alpha_map;        // occupancy extraction: [N][N][N] max of segment weights
  int occ_n, occ_pad;
};

// Layer indices: 0 .. D1-1 hidden layers of mlp1 (first: C -> W), D1: mlp1
// output (W -> W+1, sigma and the hidden feature), D1+1: mlp2 first
// (W+27 -> W), D1+2: mlp2 output (W -> 3).

template <int C, int TILE>
__device__ __forceinline__ void gather_tile(const DecodeArgs& a, long long S, long long s0, float* X0) {
  constexpr int TPS = C / 4;
  constexpr int SPP = TILE / TPS;
  const int t = threadIdx.x;
#pragma unroll 1
  for (int p = 0; p < TPS; ++p) {
    const int ls = p * SPP + t / TPS;
    const int q = t % TPS;
    const long long s = s0 + ls;
    float4 f = make_float4(0.f, 0.f, 0.f, 0.f);
    if (s < S) {
      const float* sg = a.seg + s * 6;
      const SegCorner sc = segment_corners(__ldg(sg), __ldg(sg + 1), __ldg(sg + 2), __ldg(sg + 3), __ldg(sg + 4),
                                           __ldg(sg + 5), a.nvx, a.nvy, a.nvz);
      f = integrate4(a.grid, sc, C, q, a.nvx, a.nvy);
    }
    *reinterpret_cast<float4*>(X0 + ls * (C + 4) + q * 4) = f;
  }
}

template <int C, int TILE>
__device__ __forceinline__ void scatter_tile(const DecodeArgs& a, long long S, long long s0, const float* X0) {
  constexpr int TPS = C / 4;
  constexpr int SPP = TILE / TPS;
  const int t = threadIdx.x;
#pragma unroll 1
  for (int p = 0; p < TPS; ++p) {
    const int ls = p * SPP + t / TPS;
    const int q = t % TPS;
    const long long s = s0 + ls;
    if (s < S) {
      const float* sg = a.seg + s * 6;
      const SegCorner sc = segment_corners(__ldg(sg), __ldg(sg + 1), __ldg(sg + 2), __ldg(sg + 3), __ldg(sg + 4),
                                           __ldg(sg + 5), a.nvx, a.nvy, a.nvz);
      const float4 gf = *reinterpret_cast<const float4*>(X0 + ls * (C + 4) + 4 * q);
      scatter4(a.grad_grid, sc, C, q, gf, a.nvx, a.nvy);
    }
  }
}

template <int N>
__device__ __forceinline__ void load_row(const float* src, float* dst) {
#pragma unroll
  for (int k = 0; k < N; k += 4) {
    const float4 v = *reinterpret_cast<const float4*>(src + k);
    dst[k] = v.x;
    dst[k + 1] = v.y;
    dst[k + 2] = v.z;
    dst[k + 3] = v.w;
  }
}

template <int N>
__device__ __forceinline__ void store_row(float* dst, const float* src) {
#pragma unroll
  for (int k = 0; k < N; k += 4)
    *reinterpret_cast<float4*>(dst + k) = make_float4(src[k], src[k + 1], src[k + 2], src[k + 3]);
}

__device__ __forceinline__ void load_weights(const DecodeArgs& a, float* sw) {
  for (int i = threadIdx.x; i < a.n_params / 4; i += blockDim.x)
    reinterpret_cast<float4*>(sw)[i] = __ldg(reinterpret_cast<const float4*>(a.params) + i);
}

// Forward of one segment.  x0: its feature row; H0/H1: two scratch rows of
// W+4 floats.  With STAGE, relu activations are kept for the backward:
// A[d] (input of layer d+1), A3 = (hidden, PE), A4 = relu(mlp2 hidden).
template <int C, int W, int D1, bool STAGE>
__device__ __forceinline__ float4 mlp_forward_rows(const DecodeArgs& a, const float* sw, const float* x0, int ray,
                                                   float* H0, float* H1, float* const* Arow, float* A3row,
                                                   float* A4row, bool valid) {
  float y[W + 4];
  dense_fwd_s<W, false>(sw + a.w_off[0], sw + a.b_off[0], x0, C, y);
#pragma unroll
  for (int k = 0; k < W; ++k) y[k] = valid ? fmaxf(y[k], 0.f) : 0.f;
  float* cur = STAGE ? Arow[0] : H0;
  store_row<W>(cur, y);
#pragma unroll
  for (int d = 1; d < D1; ++d) {
    dense_fwd_s<W, false>(sw + a.w_off[d], sw + a.b_off[d], cur, W, y);
#pragma unroll
    for (int k = 0; k < W; ++k) y[k] = valid ? fmaxf(y[k], 0.f) : 0.f;
    cur = STAGE ? Arow[d] : H0;
    store_row<W>(cur, y);
  }
  dense_fwd_s<W + 4, false>(sw + a.w_off[D1], sw + a.b_off[D1], cur, W, y);  // y[0] sigma, y[1..W] hidden
  const float sigma = y[0];
  float* hid = STAGE ? A3row : H1;
#pragma unroll
  for (int k = 0; k < W; k += 4)
    *reinterpret_cast<float4*>(hid + k) =
        valid ? make_float4(y[1 + k], y[2 + k], y[3 + k], y[4 + k]) : make_float4(0.f, 0.f, 0.f, 0.f);
  if (STAGE) {
    float pe[PE_PAD];
    load_row<PE_PAD>(a.pe_feat + (long long)ray * PE_PAD, pe);
#pragma unroll
    for (int k = 0; k < PE_PAD; ++k) pe[k] = valid ? pe[k] : 0.f;
    store_row<PE_PAD>(A3row + W, pe);
  }
  // mlp2 first layer: hidden @ Wt[0:W) + per-ray (bias + PE term)
  dense_fwd_s<W, false, false>(sw + a.w_off[D1 + 1], nullptr, hid, W, y);
  {
    const float* po = a.pe_out + (long long)ray * W;
#pragma unroll
    for (int k = 0; k < W; k += 4) {
      const float4 v = *reinterpret_cast<const float4*>(po + k);
      y[k] = valid ? fmaxf(y[k] + v.x, 0.f) : 0.f;
      y[k + 1] = valid ? fmaxf(y[k + 1] + v.y, 0.f) : 0.f;
      y[k + 2] = valid ? fmaxf(y[k + 2] + v.z, 0.f) : 0.f;
      y[k + 3] = valid ? fmaxf(y[k + 3] + v.w, 0.f) : 0.f;
    }
  }
  float* a4 = STAGE ? A4row : H0;
  store_row<W>(a4, y);
  float o[4];
  dense_fwd_s<4, false>(sw + a.w_off[D1 + 2], sw + a.b_off[D1 + 2], a4, W, o);
  return make_float4(sigma, sigmoidf_acc(o[0]), sigmoidf_acc(o[1]), sigmoidf_acc(o[2]));
}

template <int C, int W, int D1, int TILE>
__global__ void __launch_bounds__(TILE) decode_fwd_plain(const DecodeArgs a) {
  extern __shared__ __align__(16) float smem[];
  float* sw = smem;
  float* X0 = smem + a.n_params;
  float* H0 = X0 + TILE * (C + 4);
  float* H1 = H0 + TILE * (W + 4);
  const int t = threadIdx.x;
  load_weights(a, sw);
  __syncthreads();
  const long long S = segment_total(a.S, a.S_dev);
  const long long tiles = (S + TILE - 1) / TILE;
  for (long long tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const long long s0 = tile * TILE;
    gather_tile<C, TILE>(a, S, s0, X0);
    __syncthreads();
    const long long s = s0 + t;
    if (s < S) {
      a.out4[s] = mlp_forward_rows<C, W, D1, false>(a, sw, X0 + t * (C + 4), __ldg(a.seg_ray + s),
                                                   H0 + t * (W + 4), H1 + t * (W + 4), nullptr, nullptr, nullptr,
                                                   true);
    }
    __syncthreads();
  }
}

// dW[layer] += sum over the tile of act[s][i] * delta[s][j] (bias += delta),
// each thread owning float4 chunks of W^T rows; no two threads share a chunk.
template <int OUT4, int TILE>
__device__ __forceinline__ void accumulate_dw(float* dW, float* dB, int in, const float* act, int act_stride,
                                              const float* dl, int dl_stride) {
  constexpr int QW = OUT4 / 4;
  const int chunks = (in + 1) * QW;
  for (int c = threadIdx.x; c < chunks; c += TILE) {
    const int i = c / QW;
    const int jq = c - i * QW;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    float4* dst;
    if (i < in) {
#pragma unroll 8
      for (int s = 0; s < TILE; ++s) {
        const float x = act[s * act_stride + i];
        const float4 d = *reinterpret_cast<const float4*>(dl + s * dl_stride + 4 * jq);
        fma4(acc, x, d);
      }
      dst = reinterpret_cast<float4*>(dW + i * OUT4 + 4 * jq);
    } else {
#pragma unroll 8
      for (int s = 0; s < TILE; ++s) {
        const float4 d = *reinterpret_cast<const float4*>(dl + s * dl_stride + 4 * jq);
        acc.x += d.x;
        acc.y += d.y;
        acc.z += d.z;
        acc.w += d.w;
      }
      dst = reinterpret_cast<float4*>(dB + 4 * jq);
    }
    const float4 o = *dst;
    *dst = make_float4(o.x + acc.x, o.y + acc.y, o.z + acc.z, o.w + acc.w);
  }
}

// Shared memory of decode_bwd_plain (floats):
//   weights [n] | dW [n] | X0 [TILE][C+4] | A[0..D1) [TILE][W+4]
//   | A3 [TILE][W+28] (hidden, PE) | A4 [TILE][W+4] | DL [TILE][W+4]
template <int C, int W, int D1, int TILE>
struct BwdSmem {
  static constexpr int X0 = TILE * (C + 4);
  static constexpr int A = TILE * (W + 4);
  static constexpr int A3 = TILE * (W + PE_PAD);
  static constexpr int tile_floats = X0 + D1 * A + A3 + A + A;
};

template <int C, int W, int D1, int TILE>
__global__ void __launch_bounds__(TILE) decode_bwd_plain(const DecodeArgs a) {
  using L = BwdSmem<C, W, D1, TILE>;
  extern __shared__ __align__(16) float smem[];
  float* sw = smem;
  float* dW = smem + a.n_params;
  float* X0 = dW + a.n_params;
  float* A = X0 + L::X0;
  float* A3 = A + D1 * L::A;
  float* A4 = A3 + L::A3;
  float* DL = A4 + L::A;
  constexpr int SA = W + 4, S3 = W + PE_PAD, SX = C + 4;
  load_weights(a, sw);
  for (int i = threadIdx.x; i < a.n_params; i += TILE) dW[i] = 0.f;
  __syncthreads();
  const int t = threadIdx.x;
  float* Arow[D1];
#pragma unroll
  for (int d = 0; d < D1; ++d) Arow[d] = A + d * L::A + t * SA;
  float* A3row = A3 + t * S3;
  float* A4row = A4 + t * SA;
  float* DLrow = DL + t * SA;
  float* X0row = X0 + t * SX;
  const long long S = segment_total(a.S, a.S_dev);
  const long long tiles = (S + TILE - 1) / TILE;
  for (long long tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const long long s0 = tile * TILE;
    const long long s = s0 + t;
    const bool valid = s < S;
    gather_tile<C, TILE>(a, S, s0, X0);
    __syncthreads();
    const int ray = valid ? __ldg(a.seg_ray + s) : 0;
    const float4 c = mlp_forward_rows<C, W, D1, true>(a, sw, X0row, ray, nullptr, nullptr, Arow, A3row, A4row, valid);
    const float4 g = valid ? a.d4[s] : make_float4(0.f, 0.f, 0.f, 0.f);
    float d[W + 4];
    // mlp2 output layer (W -> 3): delta = dL/dc * sigmoid'
    d[0] = g.y * c.y * (1.f - c.y);
    d[1] = g.z * c.z * (1.f - c.z);
    d[2] = g.w * c.w * (1.f - c.w);
    d[3] = 0.f;
    store_row<4>(DLrow, d);
    __syncthreads();
    accumulate_dw<4, TILE>(dW + a.w_off[D1 + 2], dW + a.b_off[D1 + 2], W, A4, SA, DL, SA);
    __syncthreads();
    dense_bwd_input_s<4>(sw + a.w_off[D1 + 2], d, W, A4row, DLrow);  // delta of mlp2 first layer
    __syncthreads();
    accumulate_dw<W, TILE>(dW + a.w_off[D1 + 1], dW + a.b_off[D1 + 1], W + PE_DIM, A3, S3, DL, SA);
    load_row<W>(DLrow, d);
    __syncthreads();
    // mlp1 output layer: delta = (dL/dsigma, dL/dhidden)
    dense_bwd_input_s<W>(sw + a.w_off[D1 + 1], d, W, nullptr, DLrow + 1);
    DLrow[0] = g.x;
    DLrow[W + 1] = DLrow[W + 2] = DLrow[W + 3] = 0.f;
    __syncthreads();
    accumulate_dw<W + 4, TILE>(dW + a.w_off[D1], dW + a.b_off[D1], W, A + (D1 - 1) * L::A, SA, DL, SA);
    load_row<W + 4>(DLrow, d);
    __syncthreads();
    dense_bwd_input_s<W + 4>(sw + a.w_off[D1], d, W, Arow[D1 - 1], DLrow);
#pragma unroll
    for (int l = D1 - 1; l >= 1; --l) {
      __syncthreads();
      accumulate_dw<W, TILE>(dW + a.w_off[l], dW + a.b_off[l], W, A + (l - 1) * L::A, SA, DL, SA);
      load_row<W>(DLrow, d);
      __syncthreads();
      dense_bwd_input_s<W>(sw + a.w_off[l], d, W, Arow[l - 1], DLrow);
    }
    __syncthreads();
    accumulate_dw<W, TILE>(dW + a.w_off[0], dW + a.b_off[0], C, X0, SX, DL, SA);
    load_row<W>(DLrow, d);
    __syncthreads();
    dense_bwd_input_s<W>(sw + a.w_off[0], d, C, nullptr, X0row);  // dL/dfeature
    if (!valid) {
#pragma unroll
      for (int k = 0; k < C; k += 4) *reinterpret_cast<float4*>(X0row + k) = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
    scatter_tile<C, TILE>(a, S, s0, X0);
    __syncthreads();
  }
  for (int i = threadIdx.x; i < a.n_params; i += TILE)
    if (dW[i] != 0.f) atomicAdd(a.grad_params + i, dW[i]);
}

template <int C, int W, int D1, int TILE>
int launch_decode_fwd(const DecodeArgs& a, cudaStream_t st, int sms) {
  const size_t smem = (size_t)(a.n_params + TILE * (C + 4) + 2 * TILE * (W + 4)) * sizeof(float);
  auto k = decode_fwd_plain<C, W, D1, TILE>;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return DV_ERR_CUDA;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, TILE, smem);
  if (per_sm < 1) return DV_ERR_UNSUPPORTED;
  const long long tiles = (a.S + TILE - 1) / TILE;
  const long long grid = std::min<long long>(tiles, (long long)sms * per_sm);
  k<<<(unsigned)grid, TILE, smem, st>>>(a);
  DV_TRY_LAUNCH();
  return DV_OK;
}

template <int C, int W, int D1, int TILE>
int launch_decode_bwd(const DecodeArgs& a, cudaStream_t st, int sms) {
  using L = BwdSmem<C, W, D1, TILE>;
  const size_t smem = (size_t)(2 * a.n_params + L::tile_floats) * sizeof(float);
  auto k = decode_bwd_plain<C, W, D1, TILE>;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return DV_ERR_CUDA;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, TILE, smem);
  if (per_sm < 1) return DV_ERR_UNSUPPORTED;
  const long long tiles = (a.S + TILE - 1) / TILE;
  const long long grid = std::min<long long>(tiles, (long long)sms * per_sm);
  k<<<(unsigned)grid, TILE, smem, st>>>(a);
  DV_TRY_LAUNCH();
  return DV_OK;
}

// Per-variant entry points, one translation unit each.
int decode_fwd_v32c32(const DecodeArgs& a, cudaStream_t st, int sms);
int decode_bwd_v32c32(const DecodeArgs& a, cudaStream_t st, int sms);
int decode_fwd_v64c32(const DecodeArgs& a, cudaStream_t st, int sms);
int decode_bwd_v64c32(const DecodeArgs& a, cudaStream_t st, int sms);
int decode_fwd_v64c64(const DecodeArgs& a, cudaStream_t st, int sms);
int decode_bwd_v64c64(const DecodeArgs& a, cudaStream_t st, int sms);

}  // namespace dv
