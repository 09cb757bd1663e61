// Tensor-core (tcgen05) backward of the decoder for DIVeR32 (32 channels,
// width 32): per tile of 128 segments, recompute the forward on tcgen05
// keeping every layer's activations, then propagate the deltas back through
// the layers on tcgen05 (B operands = transposed weight images), accumulate
// the weight gradients on the CUDA cores, and scatter the feature gradient
// into the 8 corner rows of every segment.
//
// Shared memory (bytes; 2 CTAs per SM):
//   Bf  forward weight images   [N][K] K-major, per layer     10240
//   Bb  backward weight images  [N=in][K=out] K-major (W^T)   10240
//   bias                        forward biases (tensor-core order)
//   K   operand tile 128 x 48   K-major (forward A, backward delta)
//   R0, R1, R2, RH, R4          row-major activations: feature, relu(h0),
//                               relu(h1), (hidden | PE), relu(mlp2 hidden)
//   D   row-major delta tile 128 x 48
// The weight gradient of the CTA lives in registers: each thread owns
// 2-row x 4-column chunks of the packed torch layout (W^T [in][out4], bias),
// accumulates sum_s act[s][i] * delta[s][j] over every tile, and adds them to
// grad_params with atomics once at the end.
// Reference semantics: the autograd backward of model/diver.py:159-180.
#include "common.cuh"
#include "integrate.cuh"
#include "mlp.cuh"
#include "tc.cuh"

#include <cuda_fp16.h>

#include <algorithm>

namespace dv {

namespace bw {

constexpr int C = 32, W = 32;
constexpr int KK = W + 16;      // widest operand K (mlp1 output delta: 33 -> 48)
constexpr int SH = W + 32;      // row stride of RH: hidden (W) | PE (27) | zeros
constexpr int SD = KK;          // row stride of the delta tile
constexpr int NL = 5;
// layer: 0 (C->W), 1 (W->W), 2 (W->W+1: sigma, hidden), 3 (W+27->W), 4 (W->3)
__host__ __device__ constexpr int IN(int l) { return l == 0 ? C : (l == 3 ? W + PE_DIM : W); }
__host__ __device__ constexpr int INP(int l) { return l == 0 ? C : (l == 3 ? W + PE_PAD : W); }  // even
__host__ __device__ constexpr int OUT(int l) { return l == 2 ? W + 1 : (l == 4 ? 3 : W); }
__host__ __device__ constexpr int OUT4(int l) { return pad4(OUT(l)); }
__host__ __device__ constexpr int Q(int l) { return OUT4(l) / 4; }
__host__ __device__ constexpr int P(int l) { return INP(l) / 2 + 1; }  // pair rows incl. the bias pair
__host__ __device__ constexpr int BEGIN(int l) { return l == 0 ? 0 : BEGIN(l - 1) + P(l - 1) * Q(l - 1); }
constexpr int CHN = BEGIN(NL);
constexpr int SLOTS = (CHN + 127) / 128;

struct Args {
  const float* grid;
  int nvx, nvy, nvz;
  const float* seg;
  const int* seg_ray;
  long long S;
  const float* pe_feat;  // [B][28]
  const float* pe_out;   // [B][W]
  const float4* d4;      // [S] (dL/dsigma, dL/drgb)
  float* grad_grid;
  float* grad_params;    // packed torch layout
  int w_off[NL], b_off[NL];
  const uint8_t* wf;     // forward images
  int wf_bytes;
  const uint8_t* wb;     // backward images
  int wb_bytes;
  const float* bias;     // forward biases (tensor-core order)
  int nbias;
  int f_off[NL], f_K[NL], f_N[NL], f_bias[NL];  // forward layer table
  int b_off_img[NL], b_K[NL], b_N[NL];          // backward layer table
  int* err;
};

struct Smem {
  uint8_t* Bf;
  uint8_t* Bb;
  float* bias;
  uint8_t* K;
  uint16_t *R0, *R1, *R2, *RH, *R4, *D;
  float* stage;  // fp32 [128][C+4], aliases R1..RH
  uint64_t* bar;
  uint32_t* tslot;
};

template <int BF16>
__device__ __forceinline__ float lo16(uint32_t w) {
  if (BF16) return __uint_as_float(w << 16);
  return __half2float(__ushort_as_half((unsigned short)(w & 0xffffu)));
}
template <int BF16>
__device__ __forceinline__ float hi16(uint32_t w) {
  if (BF16) return __uint_as_float(w & 0xffff0000u);
  return __half2float(__ushort_as_half((unsigned short)(w >> 16)));
}

// Writes n (multiple of 8) values of row t at columns c0.. : into the K-major
// operand (K = kdim) when Kt != null, and into the row-major copy rowp (the
// row's start) when rowp != null.
template <int BF16>
__device__ __forceinline__ void put_row(uint8_t* Kt, int kdim, uint16_t* rowp, int t, const float* v, int n,
                                        int c0 = 0) {
#pragma unroll
  for (int c = 0; c < n; c += 8) {
    uint4 w;
    w.x = tc::pack2<BF16>(v[c], v[c + 1]);
    w.y = tc::pack2<BF16>(v[c + 2], v[c + 3]);
    w.z = tc::pack2<BF16>(v[c + 4], v[c + 5]);
    w.w = tc::pack2<BF16>(v[c + 6], v[c + 7]);
    if (Kt) *reinterpret_cast<uint4*>(Kt + tc::kmajor_offset(t, c0 + c, kdim)) = w;
    if (rowp) *reinterpret_cast<uint4*>(rowp + c0 + c) = w;
  }
}

template <int BF16>
__device__ __forceinline__ void get_row(const uint16_t* rowp, float* v, int n) {
#pragma unroll
  for (int c = 0; c < n; c += 8) {
    const uint4 w = *reinterpret_cast<const uint4*>(rowp + c);
    v[c] = lo16<BF16>(w.x);
    v[c + 1] = hi16<BF16>(w.x);
    v[c + 2] = lo16<BF16>(w.y);
    v[c + 3] = hi16<BF16>(w.y);
    v[c + 4] = lo16<BF16>(w.z);
    v[c + 5] = hi16<BF16>(w.z);
    v[c + 6] = lo16<BF16>(w.w);
    v[c + 7] = hi16<BF16>(w.w);
  }
}

template <int BF16>
__device__ __forceinline__ void issue(const uint8_t* Bimg, int K, int N, const uint8_t* At, uint32_t tmem,
                                      uint64_t* bar) {
  if (threadIdx.x == 0) {
    tc::fence_after_sync();
    const uint32_t idesc = tc::idesc_f16(128, N, BF16);
    const uint32_t a0 = tc::smem_u32(At), b0 = tc::smem_u32(Bimg);
    const uint32_t sbo = (uint32_t)(K / 8) * 128;
    for (int k = 0; k < K / 16; ++k)
      tc::mma_f16(tmem, tc::smem_desc(a0 + k * 256, 128, sbo), tc::smem_desc(b0 + k * 256, 128, sbo), idesc,
                  k > 0 ? 1u : 0u);
    tc::mma_commit(bar);
  }
}

__device__ __forceinline__ bool wait_mma(uint64_t* bar, uint32_t& phase) {
  const bool done = tc::mbar_wait_bounded(bar, phase);
  phase ^= 1u;
  tc::fence_after_sync();
  return done;
}

__device__ __forceinline__ void sync_mma() {
  tc::fence_before_sync();
  tc::fence_async_smem();
  __syncthreads();
}

// dW chunks of layer L owned by this thread: sum over the tile's segments.
template <int L, int BF16>
__device__ __forceinline__ void accumulate(float (&acc)[SLOTS][8], const uint16_t* act, int act_stride,
                                           const uint16_t* D) {
#pragma unroll
  for (int k = 0; k < SLOTS; ++k) {
    const int c = threadIdx.x + 128 * k;
    if (c < BEGIN(L) || c >= BEGIN(L + 1)) continue;
    const int local = c - BEGIN(L);
    const int p = local / Q(L), jq = local - p * Q(L);
    const bool bias_row = (2 * p == INP(L));
    float a[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] = acc[k][j];
    if (bias_row) {
#pragma unroll 4
      for (int s = 0; s < 128; ++s) {
        const uint2 d = *reinterpret_cast<const uint2*>(D + s * SD + 4 * jq);
        a[0] += lo16<BF16>(d.x);
        a[1] += hi16<BF16>(d.x);
        a[2] += lo16<BF16>(d.y);
        a[3] += hi16<BF16>(d.y);
      }
    } else {
#pragma unroll 4
      for (int s = 0; s < 128; ++s) {
        const uint32_t x = *reinterpret_cast<const uint32_t*>(act + s * act_stride + 2 * p);
        const uint2 d = *reinterpret_cast<const uint2*>(D + s * SD + 4 * jq);
        const float x0 = lo16<BF16>(x), x1 = hi16<BF16>(x);
        const float d0 = lo16<BF16>(d.x), d1 = hi16<BF16>(d.x), d2 = lo16<BF16>(d.y), d3 = hi16<BF16>(d.y);
        a[0] = fmaf(x0, d0, a[0]);
        a[1] = fmaf(x0, d1, a[1]);
        a[2] = fmaf(x0, d2, a[2]);
        a[3] = fmaf(x0, d3, a[3]);
        a[4] = fmaf(x1, d0, a[4]);
        a[5] = fmaf(x1, d1, a[5]);
        a[6] = fmaf(x1, d2, a[6]);
        a[7] = fmaf(x1, d3, a[7]);
      }
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[k][j] = a[j];
  }
}

template <int BF16>
__global__ void __launch_bounds__(128) decode_bwd_tc_kernel(const Args a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  Smem m;
  uint8_t* p = smem;
  m.Bf = p;
  p += a.wf_bytes;
  m.Bb = p;
  p += a.wb_bytes;
  m.bias = reinterpret_cast<float*>(p);
  p += a.nbias * 4;
  m.K = p;
  p += 128 * KK * 2;
  m.R0 = reinterpret_cast<uint16_t*>(p);
  p += 128 * C * 2;
  m.R1 = reinterpret_cast<uint16_t*>(p);
  m.stage = reinterpret_cast<float*>(p);
  p += 128 * W * 2;
  m.R2 = reinterpret_cast<uint16_t*>(p);
  p += 128 * W * 2;
  m.RH = reinterpret_cast<uint16_t*>(p);
  p += 128 * SH * 2;
  m.R4 = reinterpret_cast<uint16_t*>(p);
  p += 128 * W * 2;
  m.D = reinterpret_cast<uint16_t*>(p);
  p += 128 * SD * 2;
  m.bar = reinterpret_cast<uint64_t*>(p);
  m.tslot = reinterpret_cast<uint32_t*>(p + 8);

  const int t = threadIdx.x, warp = t >> 5;
  for (int i = t; i < a.wf_bytes / 16; i += 128)
    reinterpret_cast<uint4*>(m.Bf)[i] = __ldg(reinterpret_cast<const uint4*>(a.wf) + i);
  for (int i = t; i < a.wb_bytes / 16; i += 128)
    reinterpret_cast<uint4*>(m.Bb)[i] = __ldg(reinterpret_cast<const uint4*>(a.wb) + i);
  for (int i = t; i < a.nbias; i += 128) m.bias[i] = __ldg(a.bias + i);
  if (t == 0) {
    tc::mbar_init(m.bar, 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(m.tslot, 64);
    tc::tmem_relinquish();
  }
  sync_mma();
  tc::fence_after_sync();
  const uint32_t tmem = *m.tslot;
  const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
  uint32_t phase = 0;
  bool ok = true;
  float acc[SLOTS][8];
#pragma unroll
  for (int k = 0; k < SLOTS; ++k)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[k][j] = 0.f;
  float v[KK];

  const long long tiles = (a.S + 127) / 128;
  for (long long tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
    const long long s0 = tile * 128;
    const long long s = s0 + t;
    const bool valid = s < a.S;
    const int ray = valid ? __ldg(a.seg_ray + s) : 0;
    // ---- gather: feature rows (K-major operand + row-major copy) ----
    {
      constexpr int TPS = C / 4, SPP = 128 / TPS;
#pragma unroll 1
      for (int pp = 0; pp < TPS; ++pp) {
        const int ls = pp * SPP + t / TPS, q = t % TPS;
        const long long ss = s0 + ls;
        float4 f = make_float4(0.f, 0.f, 0.f, 0.f);
        if (ss < a.S) {
          const float* sg = a.seg + ss * 6;
          const SegCorner sc = segment_corners(__ldg(sg), __ldg(sg + 1), __ldg(sg + 2), __ldg(sg + 3),
                                               __ldg(sg + 4), __ldg(sg + 5), a.nvx, a.nvy, a.nvz);
          f = integrate4(a.grid, sc, C, q, a.nvx, a.nvy);
        }
        const uint2 w = make_uint2(tc::pack2<BF16>(f.x, f.y), tc::pack2<BF16>(f.z, f.w));
        *reinterpret_cast<uint2*>(m.K + tc::kmajor_offset(ls, 4 * q, C)) = w;
        *reinterpret_cast<uint2*>(m.R0 + ls * C + 4 * q) = w;
      }
    }
    sync_mma();
    // ---- forward ----
    // layer 0: relu(x0 W0^T + b0) -> R1
    issue<BF16>(m.Bf + a.f_off[0], a.f_K[0], a.f_N[0], m.K, tmem, m.bar);
    ok = __syncthreads_and(wait_mma(m.bar, phase));
    if (!ok) break;
    tc::ld_32x32b_x32(trow, v);
    tc::ld_wait();
#pragma unroll
    for (int i = 0; i < W; ++i) v[i] = fmaxf(v[i] + m.bias[a.f_bias[0] + i], 0.f);
    put_row<BF16>(m.K, W, m.R1 + t * W, t, v, W);
    sync_mma();
    // layer 1: relu(a1 W1^T + b1) -> R2
    issue<BF16>(m.Bf + a.f_off[1], a.f_K[1], a.f_N[1], m.K, tmem, m.bar);
    ok = __syncthreads_and(wait_mma(m.bar, phase));
    if (!ok) break;
    tc::ld_32x32b_x32(trow, v);
    tc::ld_wait();
#pragma unroll
    for (int i = 0; i < W; ++i) v[i] = fmaxf(v[i] + m.bias[a.f_bias[1] + i], 0.f);
    put_row<BF16>(m.K, W, m.R2 + t * W, t, v, W);
    sync_mma();
    // layer 2 (mlp1 output): hidden (columns 0..W-1) -> RH[0..W); PE -> RH[W..)
    issue<BF16>(m.Bf + a.f_off[2], a.f_K[2], a.f_N[2], m.K, tmem, m.bar);
    ok = __syncthreads_and(wait_mma(m.bar, phase));
    if (!ok) break;
    tc::ld_32x32b_x32(trow, v);
    tc::ld_wait();
#pragma unroll
    for (int i = 0; i < W; ++i) v[i] += m.bias[a.f_bias[2] + i];
    put_row<BF16>(m.K, W, m.RH + t * SH, t, v, W);
    {
      const float4* pf = reinterpret_cast<const float4*>(a.pe_feat + (long long)ray * PE_PAD);
      float pe[32];
#pragma unroll
      for (int k = 0; k < PE_PAD / 4; ++k) {
        const float4 x = __ldg(pf + k);
        pe[4 * k] = x.x;
        pe[4 * k + 1] = x.y;
        pe[4 * k + 2] = x.z;
        pe[4 * k + 3] = x.w;
      }
      pe[28] = pe[29] = pe[30] = pe[31] = 0.f;
      put_row<BF16>(nullptr, 0, m.RH + t * SH, t, pe, 32, W);
    }
    sync_mma();
    // layer 3 (mlp2 first, hidden part): relu(hid W3a^T + per-ray bias/PE) -> R4
    issue<BF16>(m.Bf + a.f_off[3], a.f_K[3], a.f_N[3], m.K, tmem, m.bar);
    ok = __syncthreads_and(wait_mma(m.bar, phase));
    if (!ok) break;
    tc::ld_32x32b_x32(trow, v);
    tc::ld_wait();
    {
      const float4* po = reinterpret_cast<const float4*>(a.pe_out + (long long)ray * W);
#pragma unroll
      for (int i = 0; i < W; i += 4) {
        const float4 x = __ldg(po + i / 4);
        v[i] = fmaxf(v[i] + x.x, 0.f);
        v[i + 1] = fmaxf(v[i + 1] + x.y, 0.f);
        v[i + 2] = fmaxf(v[i + 2] + x.z, 0.f);
        v[i + 3] = fmaxf(v[i + 3] + x.w, 0.f);
      }
    }
    put_row<BF16>(m.K, W, m.R4 + t * W, t, v, W);
    sync_mma();
    // layer 4: logits -> sigmoid -> delta4 = dL/dc * c (1 - c)
    issue<BF16>(m.Bf + a.f_off[4], a.f_K[4], a.f_N[4], m.K, tmem, m.bar);
    ok = __syncthreads_and(wait_mma(m.bar, phase));
    if (!ok) break;
    const float4 g = valid ? a.d4[s] : make_float4(0.f, 0.f, 0.f, 0.f);
    {
      float o[4];
      tc::ld_32x32b_x4(trow, o);
      tc::ld_wait();
#pragma unroll
      for (int i = 0; i < 16; ++i) v[i] = 0.f;
      const float c0 = sigmoidf_acc(o[0] + m.bias[a.f_bias[4]]);
      const float c1 = sigmoidf_acc(o[1] + m.bias[a.f_bias[4] + 1]);
      const float c2 = sigmoidf_acc(o[2] + m.bias[a.f_bias[4] + 2]);
      v[0] = g.y * c0 * (1.f - c0);
      v[1] = g.z * c1 * (1.f - c1);
      v[2] = g.w * c2 * (1.f - c2);
      put_row<BF16>(m.K, 16, m.D + t * SD, t, v, 16);
    }
    sync_mma();
    // ---- backward ----
    // through layer 4 (K = 16): dL/d relu(h3) = delta4 W4 ; delta3 = mask(R4) * that
    issue<BF16>(m.Bb + a.b_off_img[4], a.b_K[4], a.b_N[4], m.K, tmem, m.bar);
    accumulate<4, BF16>(acc, m.R4, W, m.D);
    ok = __syncthreads_and(wait_mma(m.bar, phase));
    if (!ok) break;
    {
      float r[W];
      get_row<BF16>(m.R4 + t * W, r, W);
      tc::ld_32x32b_x32(trow, v);
      tc::ld_wait();
#pragma unroll
      for (int i = 0; i < W; ++i) v[i] = (r[i] > 0.f) ? v[i] : 0.f;
      put_row<BF16>(m.K, W, m.D + t * SD, t, v, W);
    }
    sync_mma();
    // through layer 3 (K = W): d hidden = delta3 W3a ; delta of layer 2 = (dsigma, d hidden)
    issue<BF16>(m.Bb + a.b_off_img[3], a.b_K[3], a.b_N[3], m.K, tmem, m.bar);
    accumulate<3, BF16>(acc, m.RH, SH, m.D);
    ok = __syncthreads_and(wait_mma(m.bar, phase));
    if (!ok) break;
    {
      float dh[W];
      tc::ld_32x32b_x32(trow, dh);
      tc::ld_wait();
      v[0] = g.x;
#pragma unroll
      for (int i = 0; i < W; ++i) v[1 + i] = dh[i];
#pragma unroll
      for (int i = W + 1; i < KK; ++i) v[i] = 0.f;
      put_row<BF16>(m.K, KK, m.D + t * SD, t, v, KK);
    }
    sync_mma();
    // through layer 2 (K = W+16): delta1 = mask(R2) * (delta2 W2)
    issue<BF16>(m.Bb + a.b_off_img[2], a.b_K[2], a.b_N[2], m.K, tmem, m.bar);
    accumulate<2, BF16>(acc, m.R2, W, m.D);
    ok = __syncthreads_and(wait_mma(m.bar, phase));
    if (!ok) break;
    {
      float r[W];
      get_row<BF16>(m.R2 + t * W, r, W);
      tc::ld_32x32b_x32(trow, v);
      tc::ld_wait();
#pragma unroll
      for (int i = 0; i < W; ++i) v[i] = (r[i] > 0.f) ? v[i] : 0.f;
      put_row<BF16>(m.K, W, m.D + t * SD, t, v, W);
    }
    sync_mma();
    // through layer 1: delta0 = mask(R1) * (delta1 W1)
    issue<BF16>(m.Bb + a.b_off_img[1], a.b_K[1], a.b_N[1], m.K, tmem, m.bar);
    accumulate<1, BF16>(acc, m.R1, W, m.D);
    ok = __syncthreads_and(wait_mma(m.bar, phase));
    if (!ok) break;
    {
      float r[W];
      get_row<BF16>(m.R1 + t * W, r, W);
      tc::ld_32x32b_x32(trow, v);
      tc::ld_wait();
#pragma unroll
      for (int i = 0; i < W; ++i) v[i] = (r[i] > 0.f) ? v[i] : 0.f;
      put_row<BF16>(m.K, W, m.D + t * SD, t, v, W);
    }
    sync_mma();
    // through layer 0: dL/dfeature = delta0 W0 (FP32) -> staging (aliases R1..)
    issue<BF16>(m.Bb + a.b_off_img[0], a.b_K[0], a.b_N[0], m.K, tmem, m.bar);
    accumulate<0, BF16>(acc, m.R0, C, m.D);
    ok = __syncthreads_and(wait_mma(m.bar, phase));
    if (!ok) break;
    {
      tc::ld_32x32b_x32(trow, v);
      tc::ld_wait();
      float* st = m.stage + t * (C + 4);
#pragma unroll
      for (int i = 0; i < C; i += 4)
        *reinterpret_cast<float4*>(st + i) =
            valid ? make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    tc::fence_before_sync();
    __syncthreads();
    // ---- scatter dL/dfeature into the corner rows ----
    {
      constexpr int TPS = C / 4, SPP = 128 / TPS;
#pragma unroll 1
      for (int pp = 0; pp < TPS; ++pp) {
        const int ls = pp * SPP + t / TPS, q = t % TPS;
        const long long ss = s0 + ls;
        if (ss < a.S) {
          const float* sg = a.seg + ss * 6;
          const SegCorner sc = segment_corners(__ldg(sg), __ldg(sg + 1), __ldg(sg + 2), __ldg(sg + 3),
                                               __ldg(sg + 4), __ldg(sg + 5), a.nvx, a.nvy, a.nvz);
          const float4 gf = *reinterpret_cast<const float4*>(m.stage + ls * (C + 4) + 4 * q);
          scatter4(a.grad_grid, sc, C, q, gf, a.nvx, a.nvy);
        }
      }
    }
    __syncthreads();  // the next gather overwrites R0 / K; staging aliases R1..
  }
  if (!ok && t == 0 && a.err) atomicExch(a.err, 1);
  // ---- flush this CTA's weight gradient (packed torch layout) ----
#pragma unroll
  for (int k = 0; k < SLOTS; ++k) {
    const int c = t + 128 * k;
    if (c >= CHN) continue;
    int L = 0;
#pragma unroll
    for (int l = 1; l < NL; ++l)
      if (c >= BEGIN(l)) L = l;
    const int local = c - BEGIN(L);
    const int p = local / Q(L), jq = local - p * Q(L);
    float* dst;
    if (2 * p == INP(L)) {
      dst = a.grad_params + a.b_off[L] + 4 * jq;
#pragma unroll
      for (int j = 0; j < 4; ++j) atomicAdd(dst + j, acc[k][j]);
    } else {
#pragma unroll
      for (int r = 0; r < 2; ++r) {
        const int i = 2 * p + r;
        if (i >= IN(L)) continue;
        dst = a.grad_params + a.w_off[L] + i * OUT4(L) + 4 * jq;
#pragma unroll
        for (int j = 0; j < 4; ++j) atomicAdd(dst + j, acc[k][4 * r + j]);
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tmem, 64);
}

inline size_t smem_bytes(const Args& a) {
  return (size_t)a.wf_bytes + a.wb_bytes + a.nbias * 4 + 128 * KK * 2 + 128 * C * 2 + 2 * 128 * W * 2 +
         128 * SH * 2 + 128 * W * 2 + 128 * SD * 2 + 16;
}

}  // namespace bw

static int resident_bwd(const void* kernel, size_t dyn_smem) {
  cudaFuncAttributes fa{};
  if (cudaFuncGetAttributes(&fa, kernel) != cudaSuccess) return 1;
  int dev = 0, regs_sm = 65536, smem_sm = 228 * 1024;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
  cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  const int n = std::min({16, regs_sm / (std::max(fa.numRegs, 1) * 128),
                          (int)(smem_sm / (dyn_smem + fa.sharedSizeBytes + 1024)), 512 / 64});
  return std::max(n, 1);
}

}  // namespace dv

using namespace dv;

extern "C" {

int dv_decode_bwd_tc(int kind, int channels, int bf16, const void* wf, int wf_bytes, const float* bias, int nbias,
                     const int* f_layers, const void* wb, int wb_bytes, const int* b_layers, int n_layers,
                     const float* voxels, int nvx, int nvy, int nvz, const float* seg, const int* seg_ray,
                     long long n_seg, const float* pe_feat, const float* pe_out, const float* d4, float* grad_voxels,
                     float* grad_params, int* err, void* stream) {
  using namespace dv::bw;
  DV_CHECK(n_seg >= 0 && (bf16 == 0 || bf16 == 1), DV_ERR_ARG);
  DV_CHECK(kind == 32 && channels == 32 && n_layers == NL, DV_ERR_UNSUPPORTED);
  if (n_seg == 0) return DV_OK;
  DV_CHECK(wf && wb && bias && f_layers && b_layers && voxels && seg && seg_ray && pe_feat && pe_out && d4 &&
               grad_voxels && grad_params,
           DV_ERR_ARG);
  DV_CHECK(wf_bytes % 16 == 0 && wb_bytes % 16 == 0 && nbias % 4 == 0, DV_ERR_ARG);
  DV_CHECK(((uintptr_t)wf & 15) == 0 && ((uintptr_t)wb & 15) == 0 && ((uintptr_t)voxels & 15) == 0 &&
               ((uintptr_t)grad_voxels & 15) == 0 && ((uintptr_t)d4 & 15) == 0,
           DV_ERR_ARG);
  Args a{};
  a.grid = voxels;
  a.nvx = nvx;
  a.nvy = nvy;
  a.nvz = nvz;
  a.seg = seg;
  a.seg_ray = seg_ray;
  a.S = n_seg;
  a.pe_feat = pe_feat;
  a.pe_out = pe_out;
  a.d4 = reinterpret_cast<const float4*>(d4);
  a.grad_grid = grad_voxels;
  a.grad_params = grad_params;
  a.wf = reinterpret_cast<const uint8_t*>(wf);
  a.wf_bytes = wf_bytes;
  a.wb = reinterpret_cast<const uint8_t*>(wb);
  a.wb_bytes = wb_bytes;
  a.bias = bias;
  a.nbias = nbias;
  a.err = err;
  // packed torch layout offsets (same rule as dv_decoder_param_count)
  {
    int off = 0;
    const int outs[NL] = {W, W, W + 1, W, 3};
    for (int l = 0; l < NL; ++l) {
      a.w_off[l] = off;
      a.b_off[l] = off + IN(l) * pad4(outs[l]);
      off = a.b_off[l] + pad4(outs[l]);
    }
  }
  // expected operand shapes: forward (K, N) and backward (K = out padded, N = in)
  const int fK[NL] = {C, W, W, W, W}, fN[NL] = {W, W, W + 16, W, 16};
  const int bK[NL] = {W, W, W + 16, W, 16}, bN[NL] = {C, W, W, W, W};
  for (int l = 0; l < NL; ++l) {
    a.f_off[l] = f_layers[4 * l];
    a.f_K[l] = f_layers[4 * l + 1];
    a.f_N[l] = f_layers[4 * l + 2];
    a.f_bias[l] = f_layers[4 * l + 3];
    a.b_off_img[l] = b_layers[3 * l];
    a.b_K[l] = b_layers[3 * l + 1];
    a.b_N[l] = b_layers[3 * l + 2];
    DV_CHECK(a.f_K[l] == fK[l] && a.f_N[l] == fN[l] && a.b_K[l] == bK[l] && a.b_N[l] == bN[l], DV_ERR_ARG);
    DV_CHECK(a.f_off[l] % 16 == 0 && a.b_off_img[l] % 16 == 0, DV_ERR_ARG);
    DV_CHECK((long long)a.f_off[l] + (long long)fK[l] * fN[l] * 2 <= wf_bytes, DV_ERR_ARG);
    DV_CHECK((long long)a.b_off_img[l] + (long long)bK[l] * bN[l] * 2 <= wb_bytes, DV_ERR_ARG);
    DV_CHECK(a.f_bias[l] + fN[l] <= nbias, DV_ERR_ARG);
  }
  const size_t smem = smem_bytes(a);
  auto k = bf16 ? decode_bwd_tc_kernel<1> : decode_bwd_tc_kernel<0>;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return DV_ERR_CUDA;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int per_sm = resident_bwd(reinterpret_cast<const void*>(k), smem);
  const long long tiles = (n_seg + 127) / 128;
  const long long grid = std::min<long long>(tiles, (long long)sms * per_sm);
  k<<<(unsigned)grid, 128, smem, (cudaStream_t)stream>>>(a);
  DV_TRY_LAUNCH();
  return DV_OK;
}

}  // extern "C"
