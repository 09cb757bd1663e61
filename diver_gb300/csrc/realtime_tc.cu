// Tensor-core (tcgen05) form of the real-time fused decoder (mlp_eval): the
// same per-pixel contract as dv_mlp_eval — up to 8 recorded hits per call,
// the closed-form integral over the sparse feature table, the folded MLP and
// front-to-back compositing with the reference's skip (alpha < 1e-2) and
// early-termination (T < 1e-2) rules — with the folded MLP's three layers on
// the tensor cores.
// Reference: utils/mlp_evaluation/src/mlp_eval.cu:32-231 (DIVeR32) and
// utils/mlp_evaluation64/src/mlp_eval.cu:32-231 (DIVeR64).
//
// One CTA handles tiles of 128 pixels (thread t = pixel = TMEM lane t); per
// hit slot k = 0..7 the pixels' k-th hits are the rows of an M = 128 tile:
//   integral   FP32 on CUDA cores, 8 threads per row (coalesced corner rows)
//   L0         relu(integral) (DIVeR64: the integral itself) x W0^T + bias
//   L1         relu(h1) x [W2 hidden part | sigma weights]^T: h2 and sigma in
//              one MMA chain; the PE term of h2 is the pixel's own constant
//              (bias + PE weights x PE(d), FP32, computed once per pixel)
//   L2         relu(h2) x W3^T, sigmoid, compositing in hit order
// A pixel without a k-th hit (finished, or fewer hits) contributes a row of
// zeros that nobody reads.  Operands are split BF16 (every FP32 value as
// three BF16 terms, the six products whose term indices add up to at most 2),
// so the layers keep FP32-grade precision: the outputs stay within the
// intrinsic error of the reference's own FP32 kernel.
#include "common.cuh"
#include "integrate.cuh"
#include "mlp.cuh"
#include "realtime.cuh"
#include "tc.cuh"

#include <cuda_bf16.h>

#include <algorithm>

namespace dv {
namespace rtc {

// Tensor-core images of the folded layers, [N][K] in the K-major core-matrix
// layout; per layer its three terms side by side along N (term j in rows
// jN..jN+N-1, S bytes each), layers one after the other:
//   B0 [W][32]      L0 (32 -> W)
//   B1 [W + 16][W]  rows 0..W-1 the hidden part of mlp2's first layer, row W
//                   the sigma weights, the rest zero
//   B2 [16][W]      rows 0..2 the colour layer, the rest zero
template <int W>
struct Img {
  static constexpr int n0 = W, k0 = 32, n1 = W + 16, k1 = W, n2 = 16, k2 = W;
  static constexpr int s0 = n0 * k0 * 2, s1 = n1 * k1 * 2, s2 = n2 * k2 * 2;  // one term of each layer
  static constexpr int off0 = 0, off1 = off0 + 3 * s0, off2 = off1 + 3 * s1;
  static constexpr int TERM = s0 + s1 + s2;  // one term of all layers (the blob holds three)
  static constexpr int ELEMS = n0 * k0 + n1 * k1 + n2 * k2;
};

template <int W, int FIRST>
__global__ void tc_pack_kernel(const float* __restrict__ packed, uint8_t* __restrict__ blob) {
  using L = RtLayout<W, FIRST>;
  using I = Img<W>;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= I::ELEMS) return;
  int n, k, K, off, sz;
  float x;
  if (e < I::n0 * I::k0) {
    n = e / I::k0;
    k = e % I::k0;
    K = I::k0;
    off = I::off0;
    sz = I::s0;
    x = packed[L::l0_w + k * W + n];
  } else if (e < I::n0 * I::k0 + I::n1 * I::k1) {
    const int f = e - I::n0 * I::k0;
    n = f / I::k1;
    k = f % I::k1;
    K = I::k1;
    off = I::off1;
    sz = I::s1;
    x = n < W ? packed[L::l2_w + k * W + n] : (n == W ? packed[L::sig + k] : 0.f);
  } else {
    const int f = e - I::n0 * I::k0 - I::n1 * I::k1;
    n = f / I::k2;
    k = f % I::k2;
    K = I::k2;
    off = I::off2;
    sz = I::s2;
    x = n < 3 ? packed[L::l3_w + k * 4 + n] : 0.f;
  }
  const uint32_t o = off + tc::kmajor_offset(n, k, K);
  float r = x;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const __nv_bfloat16 b = __float2bfloat16_rn(r);
    *reinterpret_cast<__nv_bfloat16*>(blob + i * sz + o) = b;
    r = __fsub_rn(r, __bfloat162float(b));
  }
}

struct Args {
  int batch;
  const float* coords;   // [8][B][6]
  const float* feats;    // [F][32]
  const int* vmap;       // [(N+1)^3]
  int ms;                // N+1
  const float* params;   // aligned FP32 layout (biases, PE weights)
  const float* v;        // [B][3]
  float* rgba;           // [B][4]
  uint8_t* finish;       // [B]
  const uint8_t* wblob;  // three terms of the images
  int* err;
};

__device__ __forceinline__ int clampi(int x, int hi) { return x < 0 ? 0 : (x > hi ? hi : x); }

// One layer with three-term operands: the six products whose term indices
// add up to at most 2 as four MMAs per 16 columns of K (thread 0 issues, every
// thread waits): A0 and A1 against [B0|B1] (N = 2N) into columns 0..2N-1,
// A0 x B2 into N..2N-1 and A2 x B0 into 0..N-1.  The layer's output is the sum
// of the two column blocks (row16 / row4).
template <int K, int N>
__device__ __forceinline__ bool tc_layer3(const uint8_t* sA, uint32_t tstride, const uint8_t* sB, int boff,
                                          uint32_t tmem, uint64_t* bar, uint32_t& phase) {
  if (threadIdx.x == 0) {
    tc::fence_after_sync();
    constexpr uint32_t sbo = (K / 8) * 128;
    const uint32_t i2 = tc::idesc_f16(128, 2 * N, 1), i1 = tc::idesc_f16(128, N, 1);
    const uint64_t a0 = tc::smem_desc(tc::smem_u32(sA), 128, sbo);
    const uint64_t a1 = tc::smem_desc(tc::smem_u32(sA + tstride), 128, sbo);
    const uint64_t a2 = tc::smem_desc(tc::smem_u32(sA + 2 * tstride), 128, sbo);
    const uint64_t b01 = tc::smem_desc(tc::smem_u32(sB + boff), 128, sbo);
    const uint64_t b2 = tc::desc_plus(b01, 2 * N * K * 2);
#pragma unroll
    for (int k = 0; k < K / 16; ++k) {
      const uint32_t o = k * 256;
      tc::mma_f16(tmem, tc::desc_plus(a0, o), tc::desc_plus(b01, o), i2, k > 0 ? 1u : 0u);
      tc::mma_f16(tmem, tc::desc_plus(a1, o), tc::desc_plus(b01, o), i2, 1u);
      tc::mma_f16(tmem + N, tc::desc_plus(a0, o), tc::desc_plus(b2, o), i1, 1u);
      tc::mma_f16(tmem, tc::desc_plus(a2, o), tc::desc_plus(b01, o), i1, 1u);
    }
    tc::mma_commit(bar);
  }
  const bool done = tc::mbar_wait_bounded(bar, phase);
  if (done) phase ^= 1u;
  tc::fence_after_sync();
  return done;
}

// This thread's row of a layer's output: 16 columns from taddr plus the same
// columns of the second block n columns on (tc_layer3's two blocks).
__device__ __forceinline__ void row16(uint32_t taddr, int n, float* v) {
  float u[16];
  tc::ld_32x32b_x16(taddr, v);
  tc::ld_32x32b_x16(taddr + n, u);
  tc::ld_wait();
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] += u[i];
}

__device__ __forceinline__ void row4(uint32_t taddr, int n, float* v) {
  float u[4];
  tc::ld_32x32b_x4(taddr, v);
  tc::ld_32x32b_x4(taddr + n, u);
  tc::ld_wait();
#pragma unroll
  for (int i = 0; i < 4; ++i) v[i] += u[i];
}

// Writes n values (multiple of 8) of row t as three BF16 terms of a K-major tile with K columns.
template <int K, int n>
__device__ __forceinline__ void put_row3(uint8_t* sA, uint32_t tstride, int t, const float* v) {
#pragma unroll
  for (int c = 0; c < n; c += 8) {
    uint32_t x[3], y[3], z[3], u[3];
    tc::split_pair<3>(v[c], v[c + 1], x);
    tc::split_pair<3>(v[c + 2], v[c + 3], y);
    tc::split_pair<3>(v[c + 4], v[c + 5], z);
    tc::split_pair<3>(v[c + 6], v[c + 7], u);
    uint8_t* dst = sA + tc::kmajor_offset(t, c, K);
#pragma unroll
    for (int i = 0; i < 3; ++i) *reinterpret_cast<uint4*>(dst + i * tstride) = make_uint4(x[i], y[i], z[i], u[i]);
  }
}

// The tile's integrals, written as the A operand (three terms, K = 32
// columns): each pixel's hit k (coords and a flag in sHit, 8 floats per row)
// is integrated by 8 threads, each reading 16 bytes of every corner row, so a
// warp's loads cover 4 whole rows (coalesced).  FIRST: the integral starts
// from the pre-multiplied first layer's bias and goes through relu; rows
// without a hit are zero.
template <int FIRST>
__device__ __forceinline__ void integrate_tile(const Args& a, const float* sHit, const float* b_in, uint8_t* sA,
                                               uint32_t tstride) {
  const int t = threadIdx.x, q = t & 7;
#pragma unroll 1
  for (int p = 0; p < 8; ++p) {
    const int row = p * 16 + (t >> 3);
    const float* h = sHit + row * 8;
    float4 f = make_float4(0.f, 0.f, 0.f, 0.f);
    if (h[6] != 0.f) {
      const SegCorner sc = segment_corners(h[0], h[1], h[2], h[3], h[4], h[5], 1 << 30, 1 << 30, 1 << 30);
      float4 v[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int x = clampi(sc.x + (j & 1), a.ms - 1);
        const int yy = clampi(sc.y + ((j >> 1) & 1), a.ms - 1);
        const int z = clampi(sc.z + (j >> 2), a.ms - 1);
        const int idx = __ldg(a.vmap + ((long long)z * a.ms + yy) * a.ms + x);
        v[j] = __ldg(reinterpret_cast<const float4*>(a.feats + (long long)idx * 32) + q);
      }
      if (FIRST) f = *reinterpret_cast<const float4*>(b_in + 4 * q);
#pragma unroll
      for (int j = 0; j < 8; ++j) fma4(f, sc.w[j], v[j]);
      if (FIRST) f = make_float4(fmaxf(f.x, 0.f), fmaxf(f.y, 0.f), fmaxf(f.z, 0.f), fmaxf(f.w, 0.f));
    }
    uint32_t x[3], y[3];
    tc::split_pair<3>(f.x, f.y, x);
    tc::split_pair<3>(f.z, f.w, y);
    uint8_t* dst = sA + tc::kmajor_offset(row, 4 * q, 32);
#pragma unroll
    for (int i = 0; i < 3; ++i) *reinterpret_cast<uint2*>(dst + i * tstride) = make_uint2(x[i], y[i]);
  }
}

__device__ __forceinline__ void sync_for_mma() {
  tc::fence_before_sync();
  tc::fence_async_smem();
  __syncthreads();
}

// Bias block staged in shared memory (floats): b_in [32] | l0_b [W] | sig_b, pad [4] | l3_b [4]
template <int W>
struct Bias {
  static constexpr int b_in = 0, l0_b = 32, sig_b = 32 + W, l3_b = 36 + W, size = 40 + W;
};

// Registers capped for 4 CTAs per SM at width 32 (shared memory allows 5).
template <int W, int FIRST, int NCOLS>
__global__ void __launch_bounds__(128, W == 32 ? 4 : 1) mlp_eval_tc_kernel(const Args a) {
  using L = RtLayout<W, FIRST>;
  using I = Img<W>;
  using Bi = Bias<W>;
  constexpr int KMAX = W > 32 ? W : 32;
  constexpr uint32_t TSTRIDE = 128 * KMAX * 2;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sB = smem;
  uint8_t* sA = smem + 3 * I::TERM;
  float* sb = reinterpret_cast<float*>(sA + 3 * TSTRIDE);
  float* sHit = sb + (Bi::size + 3) / 4 * 4;  // [128][8]: this hit's coords and a hit flag per pixel
  uint64_t* bar = reinterpret_cast<uint64_t*>(sHit + 128 * 8);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 1);
  const int t = threadIdx.x, warp = t >> 5;
  for (int i = t; i < 3 * I::TERM / 16; i += 128)
    reinterpret_cast<uint4*>(sB)[i] = __ldg(reinterpret_cast<const uint4*>(a.wblob) + i);
  for (int i = t; i < Bi::size; i += 128) {
    float x = 0.f;
    if (i < 32) x = FIRST ? __ldg(a.params + L::b_in + i) : 0.f;
    else if (i < 32 + W) x = __ldg(a.params + L::l0_b + i - 32);
    else if (i == Bi::sig_b) x = __ldg(a.params + L::sig + W);
    else if (i >= Bi::l3_b && i < Bi::l3_b + 3) x = __ldg(a.params + L::l3_b + i - Bi::l3_b);
    sb[i] = x;
  }
  if (t == 0) {
    tc::mbar_init(bar, 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(tslot, NCOLS);
    tc::tmem_relinquish();
  }
  sync_for_mma();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
  uint32_t phase = 0;
  bool ok = true;
  const long long stride = (long long)a.batch * 6;
  const long long tiles = (a.batch + 127) / 128;
  for (long long tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
    const long long b = tile * 128 + t;
    const bool start = b < a.batch && !a.finish[b];
    if (!__syncthreads_or(start)) continue;
    bool alive = start, fin = false;
    float4 acc = make_float4(0.f, 0.f, 0.f, 1.f);
    float pe2[W];  // bias + PE part of mlp2's first layer for this pixel's direction (FP32)
#pragma unroll
    for (int j = 0; j < W; ++j) pe2[j] = 0.f;
    if (start) {
      acc = reinterpret_cast<const float4*>(a.rgba)[b];
      float pe[PE_PAD];
      pos_enc(__ldg(a.v + 3 * b), __ldg(a.v + 3 * b + 1), __ldg(a.v + 3 * b + 2), pe);
#pragma unroll
      for (int j = 0; j < W; ++j) pe2[j] = __ldg(a.params + L::l2_b + j);
#pragma unroll
      for (int k = 0; k < PE_DIM; ++k) {
#pragma unroll
        for (int j = 0; j < W; j += 4) {
          const float4 w = __ldg(reinterpret_cast<const float4*>(a.params + L::l2_pe + k * W + j));
          pe2[j] = fmaf(pe[k], w.x, pe2[j]);
          pe2[j + 1] = fmaf(pe[k], w.y, pe2[j + 1]);
          pe2[j + 2] = fmaf(pe[k], w.z, pe2[j + 2]);
          pe2[j + 3] = fmaf(pe[k], w.w, pe2[j + 3]);
        }
      }
    }
#pragma unroll 1
    for (int k = 0; k < 8; ++k) {
      bool hit = false;
      if (alive) {
        const float* cp = a.coords + k * stride + b * 6;
        if (__ldg(cp) < 0.f) {  // the ray left the grid before its k-th hit
          alive = false;
          fin = true;
        } else {
          hit = true;
#pragma unroll
          for (int i = 0; i < 6; ++i) sHit[t * 8 + i] = __ldg(cp + i);
        }
      }
      sHit[t * 8 + 6] = hit ? 1.f : 0.f;
      if (!__syncthreads_or(hit)) break;
      integrate_tile<FIRST>(a, sHit, sb + Bi::b_in, sA, TSTRIDE);
      sync_for_mma();
      // L0: h1 = W0 x + b0, relu
      ok = __syncthreads_and(tc_layer3<32, W>(sA, TSTRIDE, sB, I::off0, tmem, bar, phase));
      if (!ok) break;
      {
        float v[16];
#pragma unroll
        for (int c0 = 0; c0 < W; c0 += 16) {
          row16(trow + c0, I::n0, v);
#pragma unroll
          for (int i = 0; i < 16; ++i) v[i] = fmaxf(v[i] + sb[Bi::l0_b + c0 + i], 0.f);
          put_row3<W, 16>(sA + tc::kmajor_offset(0, c0, W), TSTRIDE, t, v);
        }
      }
      sync_for_mma();
      // L1: h2 (+ pixel constant) and sigma
      ok = __syncthreads_and(tc_layer3<W, W + 16>(sA, TSTRIDE, sB, I::off1, tmem, bar, phase));
      if (!ok) break;
      float alpha;
      {
        float sv[4];
        row4(trow + W, I::n1, sv);
        alpha = 1.f - expf(-fmaxf(sv[0] + sb[Bi::sig_b], 0.f));
        float v[16];
#pragma unroll
        for (int c0 = 0; c0 < W; c0 += 16) {
          row16(trow + c0, I::n1, v);
#pragma unroll
          for (int i = 0; i < 16; ++i) v[i] = fmaxf(v[i] + pe2[c0 + i], 0.f);
          put_row3<W, 16>(sA + tc::kmajor_offset(0, c0, W), TSTRIDE, t, v);
        }
      }
      sync_for_mma();
      // L2: colour logits, sigmoid, compositing (skip alpha < 1e-2, stop at T < 1e-2)
      ok = __syncthreads_and(tc_layer3<W, 16>(sA, TSTRIDE, sB, I::off2, tmem, bar, phase));
      if (!ok) break;
      {
        float o[4];
        row4(trow, I::n2, o);
        if (hit && !(alpha < 1e-2f)) {
          const float wgt = acc.w * alpha;
          acc.x += wgt * sigmoidf_acc(o[0] + sb[Bi::l3_b]);
          acc.y += wgt * sigmoidf_acc(o[1] + sb[Bi::l3_b + 1]);
          acc.z += wgt * sigmoidf_acc(o[2] + sb[Bi::l3_b + 2]);
          acc.w = acc.w * (1.f - alpha);
          if (acc.w < 1e-2f) {
            alive = false;
            fin = true;
          }
        }
      }
      tc::fence_before_sync();
      __syncthreads();  // the next hit rewrites A and TMEM
    }
    if (!ok) break;
    if (start) {
      reinterpret_cast<float4*>(a.rgba)[b] = acc;
      if (fin) a.finish[b] = 1;
    }
  }
  if (!ok && t == 0 && a.err) atomicExch(a.err, 1);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tmem, NCOLS);
}

template <int W, int FIRST>
int launch(const Args& a, cudaStream_t st) {
  using I = Img<W>;
  constexpr int NCOLS = W == 32 ? 128 : 256;  // two column blocks of the widest layer (W + 16)
  constexpr int KMAX = W > 32 ? W : 32;
  const size_t smem = 3 * (size_t)I::TERM + 3 * (size_t)128 * KMAX * 2 + (size_t)(Bias<W>::size + 3) / 4 * 16 +
                      128 * 8 * 4 + 16;
  auto k = mlp_eval_tc_kernel<W, FIRST, NCOLS>;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return DV_ERR_CUDA;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const tc::Residency res = tc::tmem_residency(reinterpret_cast<const void*>(k), smem, NCOLS, 128);
  if (res.dyn_smem != smem) {
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)res.dyn_smem) != cudaSuccess)
      return DV_ERR_CUDA;
    if (cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared) !=
        cudaSuccess)
      return DV_ERR_CUDA;
  }
  const long long tiles = (a.batch + 127) / 128;
  const long long grid = std::min<long long>(tiles, (long long)sms * res.per_sm);
  k<<<(unsigned)grid, 128, res.dyn_smem, st>>>(a);
  DV_TRY_LAUNCH();
  return DV_OK;
}

}  // namespace rtc
}  // namespace dv

using namespace dv;

extern "C" {

int dv_realtime_tc_bytes(int width) {
  if (width == 32) return 3 * rtc::Img<32>::TERM;
  if (width == 64) return 3 * rtc::Img<64>::TERM;
  return -1;
}

int dv_realtime_tc_pack(int width, const float* packed_params, void* blob, void* stream) {
  DV_CHECK((width == 32 || width == 64) && packed_params && blob, DV_ERR_ARG);
  DV_CHECK(((uintptr_t)blob & 15) == 0, DV_ERR_ARG);
  cudaStream_t st = (cudaStream_t)stream;
  if (width == 32)
    rtc::tc_pack_kernel<32, 1><<<ceil_div(rtc::Img<32>::ELEMS, 256), 256, 0, st>>>(packed_params, (uint8_t*)blob);
  else
    rtc::tc_pack_kernel<64, 0><<<ceil_div(rtc::Img<64>::ELEMS, 256), 256, 0, st>>>(packed_params, (uint8_t*)blob);
  DV_TRY_LAUNCH();
  return DV_OK;
}

int dv_mlp_eval_tc(int width, int batch_size, const float* coords, const float* voxels, const int* voxel_map,
                   int map_size, const float* packed_params, const void* tc_blob, const float* v, float* rgba,
                   uint8_t* finish, int* err, void* stream) {
  DV_CHECK((width == 32 || width == 64) && batch_size >= 0 && map_size > 0, DV_ERR_ARG);
  if (batch_size == 0) return DV_OK;
  DV_CHECK(coords && voxels && voxel_map && packed_params && tc_blob && v && rgba && finish, DV_ERR_ARG);
  DV_CHECK(((uintptr_t)voxels & 15) == 0 && ((uintptr_t)rgba & 15) == 0 && ((uintptr_t)packed_params & 15) == 0 &&
               ((uintptr_t)tc_blob & 15) == 0,
           DV_ERR_ARG);
  rtc::Args a{batch_size, coords, voxels, voxel_map, map_size, packed_params, v, rgba, finish,
              reinterpret_cast<const uint8_t*>(tc_blob), err};
  cudaStream_t st = (cudaStream_t)stream;
  return width == 32 ? rtc::launch<32, 1>(a, st) : rtc::launch<64, 0>(a, st);
}

}  // extern "C"
