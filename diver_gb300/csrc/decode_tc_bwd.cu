// Tensor-core (tcgen05) backward of the decoder for DIVeR32 (32 channels,
// width 32), BF16 operands: per tile of 128 segments, recompute the forward
// on tcgen05 keeping every layer's activations, then per layer (last first)
//   - propagate the delta:  dL/d input = delta @ W      (MMA, B = W^T image)
//   - weight gradient:      dW += delta^T @ activation  (MMA over the tile's
//     128 segments, both operands read transposed (MN-major) from the same
//     tiles; FP32 accumulators stay in TMEM for the CTA's whole life)
//   - bias gradient:        sum of the delta column (CUDA cores, registers)
// and finally scatter the feature gradient into the 8 corner rows of every
// segment with vector atomics.  Weight and bias gradients are added to the
// packed torch-layout gradient once per CTA.
//
// Shared memory (bytes; 2 CTAs per SM): forward weight images (10240),
// transposed weight images (10240), forward biases, activation tiles X0, A1,
// A2 (128 x 32), HP (128 x 64: hidden | PE | zeros), A4 (128 x 32), and the
// delta tile (128 x 128, columns past the layer's width are zero or ignored),
// all in the 8x8 core-matrix layout; FP32 staging of the feature gradient
// aliases A1..HP.  TMEM: 64 working columns + 192 columns of weight
// gradients (256).
// Reference semantics: the autograd backward of model/diver.py:159-180.
#include "common.cuh"
#include "integrate.cuh"
#include "mlp.cuh"
#include "tc.cuh"

#include <algorithm>

namespace dv {

namespace bw {

constexpr int C = 32, W = 32;
constexpr int FH = 64;          // columns of HP: hidden (W) | PE (27) | zeros
constexpr int FD = 128;         // columns of the delta tile (the weight-gradient MMA's M)
constexpr int NL = 5;
constexpr int TMEM_COLS = 256;
// layer: 0 (C->W), 1 (W->W), 2 (W->W+1: sigma, hidden), 3 (W+27->W), 4 (W->3)
__host__ __device__ constexpr int IN(int l) { return l == 0 ? C : (l == 3 ? W + PE_DIM : W); }
__host__ __device__ constexpr int OUT(int l) { return l == 2 ? W + 1 : (l == 4 ? 3 : W); }
__host__ __device__ constexpr int OUT4(int l) { return pad4(OUT(l)); }
__host__ __device__ constexpr int NIN(int l) { return l == 3 ? FH : C; }  // weight-gradient MMA N (in, padded)
__host__ __device__ constexpr int DWCOL(int l) { return l == 0 ? 64 : (l <= 3 ? DWCOL(l - 1) + NIN(l - 1) : 224); }

struct Args {
  const float* grid;
  int nvx, nvy, nvz;
  const float* seg;
  const int* seg_ray;
  long long S;           // segment count, or capacity when S_dev is set
  const int64_t* S_dev;  // optional device-held count (clamped to S)
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
  // optional: the forward's saved layer inputs (dv_decode_fwd_tc's save
  // records: X0, A1, A2, hidden, A4 tiles, 8 KiB each) and its out4; then the
  // corner rows are not gathered and the forward is not recomputed
  const uint8_t* saved;
  const float4* out4;
};
constexpr uint32_t SAVE_TILE = 128 * 2 * (C + 4 * W);  // bytes of one saved record

struct Smem {
  uint8_t *Bf, *Bb;
  float* bias;
  uint8_t *X0, *A1, *A2, *HP, *A4, *D;
  float* stage;  // fp32 [128][C+4], aliases A1..HP
  uint64_t* bar;
  uint64_t* bar_load;  // completion of the bulk loads of saved tiles
  uint32_t* tslot;
};

// Writes n (multiple of 8) values of row t at columns c0.. of a tile with F columns.
__device__ __forceinline__ void put_row(uint8_t* tile, int F, int t, const float* v, int n, int c0 = 0) {
#pragma unroll
  for (int c = 0; c < n; c += 8) {
    uint4 w;
    w.x = tc::pack2<1>(v[c], v[c + 1]);
    w.y = tc::pack2<1>(v[c + 2], v[c + 3]);
    w.z = tc::pack2<1>(v[c + 4], v[c + 5]);
    w.w = tc::pack2<1>(v[c + 6], v[c + 7]);
    *reinterpret_cast<uint4*>(tile + tc::kmajor_offset(t, c0 + c, F)) = w;
  }
}

// ReLU mask of row t (first n columns) of a BF16 tile: m[i] = act > 0.
__device__ __forceinline__ void relu_mask(const uint8_t* tile, int F, int t, float* v, int n) {
#pragma unroll
  for (int c = 0; c < n; c += 8) {
    const uint4 w = *reinterpret_cast<const uint4*>(tile + tc::kmajor_offset(t, c, F));
    const uint32_t x[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (!(__uint_as_float(x[j] << 16) > 0.f)) v[c + 2 * j] = 0.f;
      if (!(__uint_as_float(x[j] & 0xffff0000u) > 0.f)) v[c + 2 * j + 1] = 0.f;
    }
  }
}

// Forward / propagation MMA: D[128][N] = A[128 rows][K] (K-major tile with F
// columns) x B^T (B image [N][K]).
__device__ __forceinline__ void mma_rows(uint32_t d_tmem, const uint8_t* A, int F, const uint8_t* B, int K, int N) {
  const uint32_t idesc = tc::idesc_f16(128, N, 1);
  const uint32_t a0 = tc::smem_u32(A), b0 = tc::smem_u32(B);
  for (int k = 0; k < K / 16; ++k)
    tc::mma_f16(d_tmem, tc::smem_desc(a0 + k * 256, 128, (uint32_t)(F / 8) * 128),
                tc::smem_desc(b0 + k * 256, 128, (uint32_t)(K / 8) * 128), idesc, k > 0 ? 1u : 0u);
}

// Weight-gradient MMA over the tile's 128 segments: dW[128 = out][N = in] +=
// delta^T x act, both operands MN-major views of the row tiles (LBO = stride of
// 8 segments, SBO = stride of 8 features).
__device__ __forceinline__ void mma_dw(uint32_t d_tmem, const uint8_t* Dt, const uint8_t* act, int Fact, int N,
                                       bool accumulate) {
  const uint32_t idesc = tc::idesc_f16(128, N, 1) | (1u << 15) | (1u << 16);
  const uint32_t a0 = tc::smem_u32(Dt), b0 = tc::smem_u32(act);
  const uint32_t lboA = (FD / 8) * 128, lboB = (uint32_t)(Fact / 8) * 128;
  for (int k = 0; k < 8; ++k)
    tc::mma_f16(d_tmem, tc::smem_desc(a0 + k * 2 * lboA, lboA, 128), tc::smem_desc(b0 + k * 2 * lboB, lboB, 128),
                idesc, (accumulate || k > 0) ? 1u : 0u);
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

// Sum of column t of the delta tile over the 128 segments (bias gradient).
__device__ __forceinline__ float column_sum(const uint8_t* Dt, int t) {
  float s = 0.f;
#pragma unroll 8
  for (int r = 0; r < 128; ++r) {
    const uint16_t h = *reinterpret_cast<const uint16_t*>(Dt + tc::kmajor_offset(r, t, FD));
    s += __uint_as_float((uint32_t)h << 16);
  }
  return s;
}

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
  m.X0 = p;
  p += 128 * C * 2;
  m.A1 = p;
  m.stage = reinterpret_cast<float*>(p);
  p += 128 * W * 2;
  m.A2 = p;
  p += 128 * W * 2;
  m.HP = p;
  p += 128 * FH * 2;
  m.A4 = p;
  p += 128 * W * 2;
  m.D = p;
  p += 128 * FD * 2;
  m.bar = reinterpret_cast<uint64_t*>(p);
  m.bar_load = reinterpret_cast<uint64_t*>(p + 8);
  m.tslot = reinterpret_cast<uint32_t*>(p + 16);

  const int t = threadIdx.x, warp = t >> 5;
  for (int i = t; i < a.wf_bytes / 16; i += 128)
    reinterpret_cast<uint4*>(m.Bf)[i] = __ldg(reinterpret_cast<const uint4*>(a.wf) + i);
  for (int i = t; i < a.wb_bytes / 16; i += 128)
    reinterpret_cast<uint4*>(m.Bb)[i] = __ldg(reinterpret_cast<const uint4*>(a.wb) + i);
  for (int i = t; i < a.nbias; i += 128) m.bias[i] = __ldg(a.bias + i);
  for (int i = t; i < 128 * FD * 2 / 16; i += 128) reinterpret_cast<uint4*>(m.D)[i] = make_uint4(0, 0, 0, 0);
  for (int i = t; i < 128 * FH * 2 / 16; i += 128) reinterpret_cast<uint4*>(m.HP)[i] = make_uint4(0, 0, 0, 0);
  if (t == 0) {
    tc::mbar_init(m.bar, 1);
    tc::mbar_init(m.bar_load, 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(m.tslot, TMEM_COLS);
    tc::tmem_relinquish();
  }
  sync_mma();
  tc::fence_after_sync();
  const uint32_t tmem = *m.tslot;
  const uint32_t lane = (uint32_t)(warp * 32) << 16;
  const uint32_t trow = tmem + lane;
  uint32_t phase = 0, phase_load = 0;
  bool ok = true, first = true;
  float bias_acc[NL] = {0.f, 0.f, 0.f, 0.f, 0.f};
  float v[48];

  const long long S = segment_total(a.S, a.S_dev);
  const long long tiles = (S + 127) / 128;
  for (long long tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
    const long long s0 = tile * 128;
    const long long s = s0 + t;
    const bool valid = s < S;
    const int ray = valid ? __ldg(a.seg_ray + s) : 0;
    if (a.saved != nullptr) {
      // ---- saved layer inputs: bulk copies into X0, A1, A2, HP (hidden half), A4 ----
      sync_mma();  // the previous tile's reads of these buffers (and of the staging alias) are done
      if (t == 0) {
        const uint8_t* rec = a.saved + tile * (long long)SAVE_TILE;
        tc::mbar_arrive_expect_tx(m.bar_load, SAVE_TILE);
        tc::bulk_load(m.X0, rec, 128 * C * 2, m.bar_load);
        rec += 128 * C * 2;
        tc::bulk_load(m.A1, rec, 128 * W * 2, m.bar_load);
        tc::bulk_load(m.A2, rec + 128 * W * 2, 128 * W * 2, m.bar_load);
        rec += 2 * 128 * W * 2;
        // hidden tile [128][W] -> columns 0..W-1 of HP [128][FH]: one copy per 8-row group
        for (int gi = 0; gi < 16; ++gi)
          tc::bulk_load(m.HP + gi * (FH / 8) * 128, rec + gi * (W / 8) * 128, (W / 8) * 128, m.bar_load);
        rec += 128 * W * 2;
        tc::bulk_load(m.A4, rec, 128 * W * 2, m.bar_load);
      }
      {
        const float4* pf = reinterpret_cast<const float4*>(a.pe_feat + (long long)ray * PE_PAD);
#pragma unroll
        for (int k = 0; k < PE_PAD / 4; ++k) {
          const float4 x = __ldg(pf + k);
          v[4 * k] = x.x;
          v[4 * k + 1] = x.y;
          v[4 * k + 2] = x.z;
          v[4 * k + 3] = x.w;
        }
        v[28] = v[29] = v[30] = v[31] = 0.f;
        put_row(m.HP, FH, t, v, 32, W);
      }
      ok = __syncthreads_and(tc::mbar_wait_bounded(m.bar_load, phase_load));
      phase_load ^= 1u;
      if (!ok) break;
    } else {
      // ---- gather: feature rows ----
      {
        constexpr int TPS = C / 4, SPP = 128 / TPS;
  #pragma unroll 1
        for (int pp = 0; pp < TPS; ++pp) {
          const int ls = pp * SPP + t / TPS, q = t % TPS;
          const long long ss = s0 + ls;
          float4 f = make_float4(0.f, 0.f, 0.f, 0.f);
          if (ss < S) {
            const float* sg = a.seg + ss * 6;
            const SegCorner sc = segment_corners(__ldg(sg), __ldg(sg + 1), __ldg(sg + 2), __ldg(sg + 3),
                                                 __ldg(sg + 4), __ldg(sg + 5), a.nvx, a.nvy, a.nvz);
            f = integrate4(a.grid, sc, C, q, a.nvx, a.nvy);
          }
          *reinterpret_cast<uint2*>(m.X0 + tc::kmajor_offset(ls, 4 * q, C)) =
              make_uint2(tc::pack2<1>(f.x, f.y), tc::pack2<1>(f.z, f.w));
        }
      }
      sync_mma();
      // ---- forward (activations kept) ----
      if (t == 0) {
        tc::fence_after_sync();
        mma_rows(tmem, m.X0, C, m.Bf + a.f_off[0], C, W);
        tc::mma_commit(m.bar);
      }
      ok = __syncthreads_and(wait_mma(m.bar, phase));
      if (!ok) break;
      tc::ld_32x32b_x32(trow, v);
      tc::ld_wait();
  #pragma unroll
      for (int i = 0; i < W; ++i) v[i] = fmaxf(v[i] + m.bias[a.f_bias[0] + i], 0.f);
      put_row(m.A1, W, t, v, W);
      sync_mma();
      if (t == 0) {
        tc::fence_after_sync();
        mma_rows(tmem, m.A1, W, m.Bf + a.f_off[1], W, W);
        tc::mma_commit(m.bar);
      }
      ok = __syncthreads_and(wait_mma(m.bar, phase));
      if (!ok) break;
      tc::ld_32x32b_x32(trow, v);
      tc::ld_wait();
  #pragma unroll
      for (int i = 0; i < W; ++i) v[i] = fmaxf(v[i] + m.bias[a.f_bias[1] + i], 0.f);
      put_row(m.A2, W, t, v, W);
      sync_mma();
      if (t == 0) {
        tc::fence_after_sync();
        mma_rows(tmem, m.A2, W, m.Bf + a.f_off[2], W, W + 16);
        tc::mma_commit(m.bar);
      }
      ok = __syncthreads_and(wait_mma(m.bar, phase));
      if (!ok) break;
      tc::ld_32x32b_x32(trow, v);
      tc::ld_wait();
  #pragma unroll
      for (int i = 0; i < W; ++i) v[i] += m.bias[a.f_bias[2] + i];
      put_row(m.HP, FH, t, v, W);
      {
        const float4* pf = reinterpret_cast<const float4*>(a.pe_feat + (long long)ray * PE_PAD);
  #pragma unroll
        for (int k = 0; k < PE_PAD / 4; ++k) {
          const float4 x = __ldg(pf + k);
          v[4 * k] = x.x;
          v[4 * k + 1] = x.y;
          v[4 * k + 2] = x.z;
          v[4 * k + 3] = x.w;
        }
        v[28] = v[29] = v[30] = v[31] = 0.f;
        put_row(m.HP, FH, t, v, 32, W);
      }
      sync_mma();
      if (t == 0) {
        tc::fence_after_sync();
        mma_rows(tmem, m.HP, FH, m.Bf + a.f_off[3], W, W);  // hidden columns only (K = W)
        tc::mma_commit(m.bar);
      }
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
      put_row(m.A4, W, t, v, W);
      sync_mma();
      if (t == 0) {
        tc::fence_after_sync();
        mma_rows(tmem, m.A4, W, m.Bf + a.f_off[4], W, 16);
        tc::mma_commit(m.bar);
      }
      ok = __syncthreads_and(wait_mma(m.bar, phase));
      if (!ok) break;
    }
    const float4 g = valid ? a.d4[s] : make_float4(0.f, 0.f, 0.f, 0.f);
    {
      float c0, c1, c2;
      if (a.saved != nullptr) {
        const float4 oc = valid ? a.out4[s] : make_float4(0.f, 0.f, 0.f, 0.f);
        c0 = oc.y;
        c1 = oc.z;
        c2 = oc.w;
      } else {
        float o[4];
        tc::ld_32x32b_x4(trow, o);
        tc::ld_wait();
        c0 = sigmoidf_acc(o[0] + m.bias[a.f_bias[4]]);
        c1 = sigmoidf_acc(o[1] + m.bias[a.f_bias[4] + 1]);
        c2 = sigmoidf_acc(o[2] + m.bias[a.f_bias[4] + 2]);
      }
#pragma unroll
      for (int i = 0; i < 16; ++i) v[i] = 0.f;
      v[0] = g.y * c0 * (1.f - c0);
      v[1] = g.z * c1 * (1.f - c1);
      v[2] = g.w * c2 * (1.f - c2);
      put_row(m.D, FD, t, v, 16);
    }
    sync_mma();
    // ---- backward: per layer, delta propagation + weight-gradient MMA ----
    // layer 4 (delta K = 16)
    if (t == 0) {
      tc::fence_after_sync();
      mma_rows(tmem, m.D, FD, m.Bb + a.b_off_img[4], 16, W);
      mma_dw(tmem + DWCOL(4), m.D, m.A4, W, NIN(4), !first);
      tc::mma_commit(m.bar);
    }
    if (t < OUT(4)) bias_acc[4] += column_sum(m.D, t);
    ok = __syncthreads_and(wait_mma(m.bar, phase));
    if (!ok) break;
    tc::ld_32x32b_x32(trow, v);
    tc::ld_wait();
    relu_mask(m.A4, W, t, v, W);
    put_row(m.D, FD, t, v, W);  // delta3
    sync_mma();
    // layer 3 (mlp2 first; delta K = W): d hidden; weight gradient over (hidden | PE)
    if (t == 0) {
      tc::fence_after_sync();
      mma_rows(tmem, m.D, FD, m.Bb + a.b_off_img[3], W, W);
      mma_dw(tmem + DWCOL(3), m.D, m.HP, FH, NIN(3), !first);
      tc::mma_commit(m.bar);
    }
    if (t < OUT(3)) bias_acc[3] += column_sum(m.D, t);
    ok = __syncthreads_and(wait_mma(m.bar, phase));
    if (!ok) break;
    {
      float dh[32];
      tc::ld_32x32b_x32(trow, dh);
      tc::ld_wait();
      v[0] = g.x;
#pragma unroll
      for (int i = 0; i < W; ++i) v[1 + i] = dh[i];
#pragma unroll
      for (int i = W + 1; i < 48; ++i) v[i] = 0.f;
      put_row(m.D, FD, t, v, 48);  // delta of layer 2: (dsigma, d hidden)
    }
    sync_mma();
    // layer 2 (mlp1 output; delta K = W + 16)
    if (t == 0) {
      tc::fence_after_sync();
      mma_rows(tmem, m.D, FD, m.Bb + a.b_off_img[2], W + 16, W);
      mma_dw(tmem + DWCOL(2), m.D, m.A2, W, NIN(2), !first);
      tc::mma_commit(m.bar);
    }
    if (t < OUT(2)) bias_acc[2] += column_sum(m.D, t);
    ok = __syncthreads_and(wait_mma(m.bar, phase));
    if (!ok) break;
    tc::ld_32x32b_x32(trow, v);
    tc::ld_wait();
    relu_mask(m.A2, W, t, v, W);
    put_row(m.D, FD, t, v, W);  // delta1
    sync_mma();
    // layer 1
    if (t == 0) {
      tc::fence_after_sync();
      mma_rows(tmem, m.D, FD, m.Bb + a.b_off_img[1], W, W);
      mma_dw(tmem + DWCOL(1), m.D, m.A1, W, NIN(1), !first);
      tc::mma_commit(m.bar);
    }
    if (t < OUT(1)) bias_acc[1] += column_sum(m.D, t);
    ok = __syncthreads_and(wait_mma(m.bar, phase));
    if (!ok) break;
    tc::ld_32x32b_x32(trow, v);
    tc::ld_wait();
    relu_mask(m.A1, W, t, v, W);
    put_row(m.D, FD, t, v, W);  // delta0
    sync_mma();
    // layer 0: dL/dfeature (FP32) -> staging (aliases A1..HP, no longer read)
    if (t == 0) {
      tc::fence_after_sync();
      mma_rows(tmem, m.D, FD, m.Bb + a.b_off_img[0], W, C);
      mma_dw(tmem + DWCOL(0), m.D, m.X0, C, NIN(0), !first);
      tc::mma_commit(m.bar);
    }
    if (t < OUT(0)) bias_acc[0] += column_sum(m.D, t);
    ok = __syncthreads_and(wait_mma(m.bar, phase));
    if (!ok) break;
    first = false;
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
        if (ss < S) {
          const float* sg = a.seg + ss * 6;
          const SegCorner sc = segment_corners(__ldg(sg), __ldg(sg + 1), __ldg(sg + 2), __ldg(sg + 3),
                                               __ldg(sg + 4), __ldg(sg + 5), a.nvx, a.nvy, a.nvz);
          const float4 gf = *reinterpret_cast<const float4*>(m.stage + ls * (C + 4) + 4 * q);
          scatter4(a.grad_grid, sc, C, q, gf, a.nvx, a.nvy);
        }
      }
    }
    tc::fence_before_sync();
    __syncthreads();  // the next gather overwrites X0; staging aliases A1..HP
    tc::fence_after_sync();
  }
  if (!ok && t == 0 && a.err) atomicExch(a.err, 1);
  // ---- flush: weight gradients from TMEM (row o = out index = this thread's lane) ----
  if (ok && !first) {
#pragma unroll
    for (int l = 0; l < NL; ++l) {
      const int o = t;
#pragma unroll
      for (int c0 = 0; c0 < NIN(l); c0 += 32) {
        tc::ld_32x32b_x32(tmem + lane + DWCOL(l) + c0, v);
        tc::ld_wait();
        if (o < OUT(l)) {
#pragma unroll
          for (int i = 0; i < 32; ++i)
            if (c0 + i < IN(l)) atomicAdd(a.grad_params + a.w_off[l] + (c0 + i) * OUT4(l) + o, v[i]);
        }
      }
      if (o < OUT(l)) atomicAdd(a.grad_params + a.b_off[l] + o, bias_acc[l]);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tmem, TMEM_COLS);
}

inline size_t smem_bytes(const Args& a) {
  return (size_t)a.wf_bytes + a.wb_bytes + a.nbias * 4 + 128 * C * 2 + 2 * 128 * W * 2 + 128 * FH * 2 +
         128 * W * 2 + 128 * FD * 2 + 32;
}

}  // namespace bw

}  // namespace dv

using namespace dv;

extern "C" {

int dv_decode_bwd_tc(int kind, int channels, int bf16, const void* wf, int wf_bytes, const float* bias, int nbias,
                     const int* f_layers, const void* wb, int wb_bytes, const int* b_layers, int n_layers,
                     const float* voxels, int nvx, int nvy, int nvz, const float* seg, const int* seg_ray,
                     long long n_seg, const int64_t* n_seg_dev, const float* pe_feat, const float* pe_out,
                     const float* d4, const void* saved, long long saved_bytes, const float* out4,
                     float* grad_voxels, float* grad_params, int* err, void* stream) {
  using namespace dv::bw;
  DV_CHECK(n_seg >= 0 && (bf16 == 0 || bf16 == 1), DV_ERR_ARG);
  DV_CHECK(kind == 32 && channels == 32 && n_layers == NL && bf16 == 1, DV_ERR_UNSUPPORTED);
  if (n_seg == 0) return DV_OK;
  DV_CHECK(wf && wb && bias && f_layers && b_layers && voxels && seg && seg_ray && pe_feat && pe_out && d4 &&
               grad_voxels && grad_params,
           DV_ERR_ARG);
  DV_CHECK(wf_bytes % 16 == 0 && wb_bytes % 16 == 0 && nbias % 4 == 0, DV_ERR_ARG);
  DV_CHECK(((uintptr_t)wf & 15) == 0 && ((uintptr_t)wb & 15) == 0 && ((uintptr_t)voxels & 15) == 0 &&
               ((uintptr_t)grad_voxels & 15) == 0 && ((uintptr_t)d4 & 15) == 0,
           DV_ERR_ARG);
  if (saved != nullptr) {
    DV_CHECK(out4 != nullptr && ((uintptr_t)saved & 15) == 0 && ((uintptr_t)out4 & 15) == 0, DV_ERR_ARG);
    DV_CHECK((n_seg + 127) / 128 * (long long)SAVE_TILE <= saved_bytes, DV_ERR_ARG);
  }
  Args a{};
  a.saved = reinterpret_cast<const uint8_t*>(saved);
  a.out4 = reinterpret_cast<const float4*>(out4);
  a.grid = voxels;
  a.nvx = nvx;
  a.nvy = nvy;
  a.nvz = nvz;
  a.seg = seg;
  a.seg_ray = seg_ray;
  a.S = n_seg;
  a.S_dev = n_seg_dev;
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
  auto k = decode_bwd_tc_kernel;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return DV_ERR_CUDA;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const tc::Residency res = tc::tmem_residency(reinterpret_cast<const void*>(k), smem, bw::TMEM_COLS, 128);
  if (res.dyn_smem != smem) {
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)res.dyn_smem) != cudaSuccess)
      return DV_ERR_CUDA;
    if (cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared) !=
        cudaSuccess)
      return DV_ERR_CUDA;
  }
  const long long tiles = (n_seg + 127) / 128;
  const long long grid = std::min<long long>(tiles, (long long)sms * res.per_sm);
  k<<<(unsigned)grid, 128, res.dyn_smem, (cudaStream_t)stream>>>(a);
  DV_TRY_LAUNCH();
  return DV_OK;
}

}  // extern "C"
