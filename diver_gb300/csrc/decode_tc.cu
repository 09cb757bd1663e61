// Tensor-core (tcgen05) decoder forward for the training / offline path.
//
// One CTA = 128 threads = one tile of 128 segments = the 128 TMEM lanes of
// an M=128 MMA.  Per tile:
//   gather  C/4 threads per segment read the 8 corner rows (coalesced float4),
//           integrate in FP32 and write the feature row as BF16/FP16 straight
//           into the K-major A operand tile in shared memory
//   layers  each Linear layer is one chain of K/16 tcgen05.mma (A and B from
//           shared memory, FP32 accumulators in TMEM), committed to an
//           mbarrier; thread t then reads its row (TMEM lane t), adds the bias,
//           applies ReLU and writes the next A tile row
//   output  sigma (FP32) and sigmoid(rgb) per segment
// The decoder's weights (all layers, B operands in the same K-major layout)
// and biases stay in shared memory for the CTA's lifetime; the grid is
// persistent over tiles and sized so TMEM never oversubscribes.
// Reference semantics: model/diver.py:159-180 (mlp1, PE, mlp2, sigmoid).
#include "common.cuh"
#include "integrate.cuh"
#include "mlp.cuh"
#include "tc.cuh"

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>

namespace dv {

constexpr int TC_MAX_LAYERS = 5;

struct TcLayer {
  int b_off;     // byte offset of the layer's B image in the weight blob
  int K, N;      // padded: K % 16 == 0, N % 16 == 0
  int bias_off;  // float offset of the layer's bias (N entries)
  int s_off;     // split form: byte offset of the layer's [3 x N][K] image (terms side by side) in shared memory
};

struct TcArgs {
  const float* grid;
  const uint16_t* grid16;  // optional BF16/FP16 copy of the grid (same layout); used when non-null
  int nvx, nvy, nvz;
  const float* seg;
  const int* seg_ray;
  long long S;           // segment count, or capacity when S_dev is set
  const int64_t* S_dev;  // optional device-held count (clamped to S)
  const float* pe_out;  // [B][W]: bias + PE part of mlp2's first layer (FP32)
  float4* out4;
  const uint8_t* wblob;
  int wbytes;  // bytes of one term's weight images (multiple of 16); TERMS terms follow each other
  const float* bias;
  int nbias;   // multiple of 4
  TcLayer L[TC_MAX_LAYERS];
  int* err;    // set to 1 if an MMA completion wait timed out
  uint8_t* save;       // optional: every layer's input tile, per 128-segment tile (training)
  int save_off[TC_MAX_LAYERS];  // byte offset of layer l's input tile inside a tile's record
  int save_bytes;      // bytes per tile record (sum of 256 * K over the layers)
};

// Address of term i of element (r, c) of an A tile with K columns.  One term:
// a [128][K] K-major tile at sA.  Three terms: terms 0 and 1 side by side in
// one [128][2K] tile at sA (columns i * K + c; the two-term copy of the layer
// input that the training backward reads back, saved with one bulk copy),
// term 2 in a [128][K] tile of its own at sA + 2 * tstride.
template <int TERMS>
__device__ __forceinline__ uint8_t* a_term(uint8_t* sA, uint32_t tstride, int r, int c, int K, int i) {
  if constexpr (TERMS == 1) return sA + tc::kmajor_offset(r, c, K);
  return i < 2 ? sA + tc::kmajor_offset(r, i * K + c, 2 * K) : sA + 2 * tstride + tc::kmajor_offset(r, c, K);
}

// Gather from the FP32 grid: C/4 threads per segment, each integrating 4
// channels; the feature row goes to the A tile as TERMS operand terms (a_term).
template <int C, int BF16, int TERMS>
__device__ __forceinline__ void gather_tile_lp(const TcArgs& a, long long S, long long s0, uint8_t* sA,
                                               uint32_t tstride) {
  constexpr int TPS = C / 4;
  constexpr int SPP = 128 / TPS;
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
    if constexpr (TERMS == 1) {
      *reinterpret_cast<uint2*>(a_term<1>(sA, tstride, ls, 4 * q, C, 0)) =
          make_uint2(tc::pack2<BF16>(f.x, f.y), tc::pack2<BF16>(f.z, f.w));
    } else {
      uint32_t x[TERMS], y[TERMS];
      tc::split_pair<TERMS>(f.x, f.y, x);
      tc::split_pair<TERMS>(f.z, f.w, y);
#pragma unroll
      for (int i = 0; i < TERMS; ++i)
        *reinterpret_cast<uint2*>(a_term<TERMS>(sA, tstride, ls, 4 * q, C, i)) = make_uint2(x[i], y[i]);
    }
  }
}

// The split form's gather (FP32 grid, three operand terms): the same passes as
// gather_tile_lp, two at a time, so each thread has 16 corner-row loads in
// flight.  The split kernel runs 4 CTAs per SM (its shared memory), so the
// registers this takes cost no residency; the single-term kernels keep the
// one-pass gather (their residency is register-bound).
template <int C, int TERMS>
__device__ __forceinline__ void gather_tile_lp_x2(const TcArgs& a, long long S, long long s0, uint8_t* sA,
                                                  uint32_t tstride) {
  constexpr int TPS = C / 4;
  constexpr int SPP = 128 / TPS;
  static_assert(TPS % 2 == 0, "passes are taken in pairs");
  const int t = threadIdx.x;
  const int q = t % TPS;
#pragma unroll 1
  for (int p = 0; p < TPS; p += 2) {
    SegCorner sc[2];
    float4 v[2][8];
    bool in[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const long long s = s0 + (p + u) * SPP + t / TPS;
      in[u] = s < S;
      if (in[u]) {
        const float* sg = a.seg + s * 6;
        sc[u] = segment_corners(__ldg(sg), __ldg(sg + 1), __ldg(sg + 2), __ldg(sg + 3), __ldg(sg + 4), __ldg(sg + 5),
                                a.nvx, a.nvy, a.nvz);
#pragma unroll
        for (int j = 0; j < 8; ++j) v[u][j] = ldg4(a.grid + corner_row(sc[u], j, a.nvx, a.nvy) * C + q * 4);
      }
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      float4 f = make_float4(0.f, 0.f, 0.f, 0.f);
      if (in[u]) {
#pragma unroll
        for (int j = 0; j < 8; ++j) fma4(f, sc[u].w[j], v[u][j]);
      }
      uint32_t x[TERMS], y[TERMS];
      tc::split_pair<TERMS>(f.x, f.y, x);
      tc::split_pair<TERMS>(f.z, f.w, y);
#pragma unroll
      for (int i = 0; i < TERMS; ++i)
        *reinterpret_cast<uint2*>(a_term<TERMS>(sA, tstride, (p + u) * SPP + t / TPS, 4 * q, C, i)) =
            make_uint2(x[i], y[i]);
    }
  }
}

template <int BF16>
__device__ __forceinline__ void unpack8(const uint4 w, float* f) {
  const uint32_t x[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    if (BF16) {
      f[2 * j] = __uint_as_float(x[j] << 16);
      f[2 * j + 1] = __uint_as_float(x[j] & 0xffff0000u);
    } else {
      f[2 * j] = __half2float(__ushort_as_half((unsigned short)(x[j] & 0xffffu)));
      f[2 * j + 1] = __half2float(__ushort_as_half((unsigned short)(x[j] >> 16)));
    }
  }
}

// Gather from the 16-bit copy of the grid: C/8 threads per segment, each
// reading 16 bytes (8 channels) of every corner row; the integral is FP32.
template <int C, int BF16>
__device__ __forceinline__ void gather_tile_16(const TcArgs& a, long long S, long long s0, uint8_t* sA) {
  constexpr int TPS = C / 8;
  constexpr int SPP = 128 / TPS;
  const int t = threadIdx.x;
#pragma unroll 1
  for (int p = 0; p < TPS; ++p) {
    const int ls = p * SPP + t / TPS;
    const int q = t % TPS;
    const long long s = s0 + ls;
    float f[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (s < S) {
      const float* sg = a.seg + s * 6;
      const SegCorner sc = segment_corners(__ldg(sg), __ldg(sg + 1), __ldg(sg + 2), __ldg(sg + 3), __ldg(sg + 4),
                                           __ldg(sg + 5), a.nvx, a.nvy, a.nvz);
      uint4 w[8];
#pragma unroll
      for (int j = 0; j < 8; ++j)
        w[j] = __ldg(reinterpret_cast<const uint4*>(a.grid16 + corner_row(sc, j, a.nvx, a.nvy) * C) + q);
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        float g[8];
        unpack8<BF16>(w[j], g);
#pragma unroll
        for (int k = 0; k < 8; ++k) f[k] = fmaf(sc.w[j], g[k], f[k]);
      }
    }
    uint4 o;
    o.x = tc::pack2<BF16>(f[0], f[1]);
    o.y = tc::pack2<BF16>(f[2], f[3]);
    o.z = tc::pack2<BF16>(f[4], f[5]);
    o.w = tc::pack2<BF16>(f[6], f[7]);
    *reinterpret_cast<uint4*>(sA + tc::kmajor_offset(ls, 8 * q, C)) = o;
  }
}

// Issues one layer's MMA chain (thread 0) and waits for it (all threads).
// With TERMS = 3 the A tile and the weight images are three BF16 terms each
// and the chain sums the six products whose term indices add up to at most 2
// (FP32-grade products) in four MMAs per 16 columns of K: A0 and A1 against
// the weight terms [W0|W1] side by side (N = 2N), A0 x W2 into columns
// N..2N-1 and A2 x W0 into columns 0..N-1; the layer's output is the sum of
// the two column blocks (acc_row / acc_row4).  A tcgen05.mma costs about the
// same at N = 2N as at N, so this is two MMAs fewer per K step.  With `save`, thread 0 also copies the layer's input
// tile (the A operand, 256 * K bytes; with TERMS = 3 the [128][2K] tile of its
// first two terms, a two-term split of the same values) to global memory by a
// bulk async copy and, before the caller's barrier lets anyone overwrite A,
// waits until that copy has read it.
template <int BF16, int TERMS>
__device__ __forceinline__ bool tc_layer(const TcLayer& L, const uint8_t* sB, uint32_t wterm, const uint8_t* sA,
                                         uint32_t tstride, uint32_t tmem, uint64_t* bar, uint32_t& phase,
                                         uint8_t* save = nullptr) {
  if (threadIdx.x == 0) {
    tc::fence_after_sync();
    if (save != nullptr) {
      tc::bulk_store(save, sA, (uint32_t)L.K * 256u * (TERMS > 1 ? 2u : 1u));
      tc::bulk_commit();
    }
    const uint32_t sbo = (uint32_t)(L.K / 8) * 128;
    if constexpr (TERMS == 1) {
      const uint32_t idesc = tc::idesc_f16(128, L.N, BF16);
      const uint32_t a0 = tc::smem_u32(sA), b0 = tc::smem_u32(sB + L.b_off);
      for (int k = 0; k < L.K / 16; ++k)
        tc::mma_f16(tmem, tc::smem_desc(a0 + k * 256, 128, sbo), tc::smem_desc(b0 + k * 256, 128, sbo), idesc,
                    k > 0 ? 1u : 0u);
    } else {
      // A terms (a_term's layout): 0 and 1 are K-column slices of the [128][2K] tile, 2 its own tile
      const uint64_t a0 = tc::smem_desc(tc::smem_u32(sA), 128, 2 * sbo);
      const uint64_t a1 = tc::desc_plus(a0, (uint32_t)(L.K / 8) * 128);
      const uint64_t a2 = tc::smem_desc(tc::smem_u32(sA + 2 * tstride), 128, sbo);
      // weights [W0|W1|W2] along N (rows): [W0|W1] is the first 2N rows, W0 the first N
      const uint64_t b01 = tc::smem_desc(tc::smem_u32(sB + L.s_off), 128, sbo);
      const uint64_t b2 = tc::desc_plus(b01, (uint32_t)(2 * L.N * L.K * 2));
      const uint32_t i2 = tc::idesc_f16(128, 2 * L.N, 1), i1 = tc::idesc_f16(128, L.N, 1);
      for (int k = 0; k < L.K / 16; ++k) {
        const uint32_t o = (uint32_t)k * 256;
        tc::mma_f16(tmem, tc::desc_plus(a0, o), tc::desc_plus(b01, o), i2, k > 0 ? 1u : 0u);
        tc::mma_f16(tmem, tc::desc_plus(a1, o), tc::desc_plus(b01, o), i2, 1u);
        tc::mma_f16(tmem + L.N, tc::desc_plus(a0, o), tc::desc_plus(b2, o), i1, 1u);
        tc::mma_f16(tmem, tc::desc_plus(a2, o), tc::desc_plus(b01, o), i1, 1u);
      }
    }
    tc::mma_commit(bar);
  }
  const bool done = tc::mbar_wait_bounded(bar, phase);
  phase ^= 1u;
  tc::fence_after_sync();
  if (save != nullptr && threadIdx.x == 0) tc::bulk_wait_read();
  return done;
}

// Epilogue columns per pass: 32, or 16 for the split form, whose rows are the
// sum of two TMEM column blocks (registers: its kernel runs 4 CTAs per SM).
template <int TERMS>
constexpr int EPI_COLS = TERMS == 1 ? 32 : 16;

// This thread's row of a layer's output, EPI_COLS columns from taddr; with
// TERMS = 3 the sum of tc_layer's two column blocks (the second n columns on).
template <int TERMS>
__device__ __forceinline__ void acc_row(uint32_t taddr, int n, float* v) {
  if constexpr (TERMS == 1) {
    tc::ld_32x32b_x32(taddr, v);
    tc::ld_wait();
  } else {
    float u[16];
    tc::ld_32x32b_x16(taddr, v);
    tc::ld_32x32b_x16(taddr + n, u);
    tc::ld_wait();
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] += u[i];
  }
}

// Same for 4 columns.
template <int TERMS>
__device__ __forceinline__ void acc_row4(uint32_t taddr, int n, float* v) {
  tc::ld_32x32b_x4(taddr, v);
  if constexpr (TERMS > 1) {
    float u[4];
    tc::ld_32x32b_x4(taddr + n, u);
    tc::ld_wait();
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] += u[i];
  } else {
    tc::ld_wait();
  }
}

// Writes EPI_COLS values (columns c0.. of the next layer's input) of row t,
// as TERMS operand terms (a_term's layout).
template <int BF16, int TERMS>
__device__ __forceinline__ void store_row(uint8_t* sA, uint32_t tstride, int t, int c0, int K, const float* v) {
#pragma unroll
  for (int j = 0; j < EPI_COLS<TERMS> / 8; ++j) {
    if constexpr (TERMS == 1) {
      uint4 w;
      w.x = tc::pack2<BF16>(v[8 * j + 0], v[8 * j + 1]);
      w.y = tc::pack2<BF16>(v[8 * j + 2], v[8 * j + 3]);
      w.z = tc::pack2<BF16>(v[8 * j + 4], v[8 * j + 5]);
      w.w = tc::pack2<BF16>(v[8 * j + 6], v[8 * j + 7]);
      *reinterpret_cast<uint4*>(a_term<1>(sA, tstride, t, c0 + 8 * j, K, 0)) = w;
    } else {
      uint32_t x[TERMS], y[TERMS], z[TERMS], u[TERMS];
      tc::split_pair<TERMS>(v[8 * j + 0], v[8 * j + 1], x);
      tc::split_pair<TERMS>(v[8 * j + 2], v[8 * j + 3], y);
      tc::split_pair<TERMS>(v[8 * j + 4], v[8 * j + 5], z);
      tc::split_pair<TERMS>(v[8 * j + 6], v[8 * j + 7], u);
#pragma unroll
      for (int i = 0; i < TERMS; ++i)
        *reinterpret_cast<uint4*>(a_term<TERMS>(sA, tstride, t, c0 + 8 * j, K, i)) = make_uint4(x[i], y[i], z[i], u[i]);
    }
  }
}

__device__ __forceinline__ void sync_for_mma() {
  tc::fence_before_sync();
  tc::fence_async_smem();
  __syncthreads();
}

// NCOLS: TMEM columns (>= widest N, power of two >= 32).  TERMS: operand
// terms (1: BF16 or FP16 operands; 3: FP32 values as three BF16 terms, six
// products per layer, FP32-grade; BF16 only and read from the FP32 grid).
// Registers per thread are capped to the residency the other resources allow:
// 8 CTAs per SM for the single-term forms (TMEM), 4 for the DIVeR32 split
// form (shared memory; its two-pass gather would otherwise take 3).
template <int C, int W, int D1, int BF16, int NCOLS, int TERMS>
__global__ void __launch_bounds__(128, TERMS == 1 ? 8 : ((C == 32 && W == 32) ? 4 : 1)) decode_fwd_tc(const TcArgs a) {
  constexpr int KMAX = C > W ? C : W;
  constexpr uint32_t TSTRIDE = 128 * KMAX * 2;  // bytes between the A tile's terms
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sB = smem;
  float* sBias = reinterpret_cast<float*>(smem + TERMS * a.wbytes);
  uint8_t* sA = reinterpret_cast<uint8_t*>(sBias + a.nbias);
  uint64_t* bar = reinterpret_cast<uint64_t*>(sA + TERMS * TSTRIDE);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 1);
  const int t = threadIdx.x, warp = t >> 5;
  if constexpr (TERMS == 1) {
    for (int i = t; i < a.wbytes / 16; i += 128)
      reinterpret_cast<uint4*>(sB)[i] = __ldg(reinterpret_cast<const uint4*>(a.wblob) + i);
  } else {
    // the images regrouped layer by layer, the three terms side by side along N
#pragma unroll 1
    for (int l = 0; l < D1 + 3; ++l) {
      const TcLayer& L = a.L[l];
      const int img16 = L.N * L.K * 2 / 16;
      for (int i = t; i < 3 * img16; i += 128) {
        const int j = i / img16, o = i % img16;
        reinterpret_cast<uint4*>(sB + L.s_off)[i] =
            __ldg(reinterpret_cast<const uint4*>(a.wblob + (size_t)j * a.wbytes + L.b_off) + o);
      }
    }
  }
  for (int i = t; i < a.nbias; i += 128) sBias[i] = __ldg(a.bias + i);
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
  const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);  // this warp's TMEM lanes
  const uint32_t wterm = (uint32_t)a.wbytes;
  uint32_t phase = 0;
  bool ok = true;
  const long long S = segment_total(a.S, a.S_dev);
  const long long tiles = (S + 127) / 128;
  for (long long tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
    const long long s0 = tile * 128;
    const long long s = s0 + t;
    const bool valid = s < S;
    uint8_t* rec = a.save ? a.save + tile * (long long)a.save_bytes : nullptr;
#define DV_SAVE(l) (rec ? rec + a.save_off[l] : nullptr)
    if constexpr (TERMS > 1) {
      gather_tile_lp_x2<C, TERMS>(a, S, s0, sA, TSTRIDE);
    } else {
      if (a.grid16)
        gather_tile_16<C, BF16>(a, S, s0, sA);
      else
        gather_tile_lp<C, BF16, TERMS>(a, S, s0, sA, TSTRIDE);
    }
    sync_for_mma();
    float v[32];
    // mlp1 hidden layers: D = relu(A W^T + b)
#pragma unroll 1
    for (int l = 0; l < D1 && ok; ++l) {
      ok = tc_layer<BF16, TERMS>(a.L[l], sB, wterm, sA, TSTRIDE, tmem, bar, phase, DV_SAVE(l));
      ok = __syncthreads_and(ok);
      if (!ok) break;
#pragma unroll
      for (int c0 = 0; c0 < W; c0 += EPI_COLS<TERMS>) {
        acc_row<TERMS>(trow + c0, a.L[l].N, v);
#pragma unroll
        for (int i = 0; i < EPI_COLS<TERMS>; ++i) v[i] = fmaxf(v[i] + sBias[a.L[l].bias_off + c0 + i], 0.f);
        store_row<BF16, TERMS>(sA, TSTRIDE, t, c0, W, v);
      }
      sync_for_mma();
    }
    if (!ok) break;
    // mlp1 output: columns 0..W-1 hidden (no activation), column W sigma
    ok = __syncthreads_and(tc_layer<BF16, TERMS>(a.L[D1], sB, wterm, sA, TSTRIDE, tmem, bar, phase, DV_SAVE(D1)));
    if (!ok) break;
    float sigma;
    {
      float sv[4];
      acc_row4<TERMS>(trow + W, a.L[D1].N, sv);
      sigma = sv[0] + sBias[a.L[D1].bias_off + W];
    }
#pragma unroll
    for (int c0 = 0; c0 < W; c0 += EPI_COLS<TERMS>) {
      acc_row<TERMS>(trow + c0, a.L[D1].N, v);
#pragma unroll
      for (int i = 0; i < EPI_COLS<TERMS>; ++i) v[i] += sBias[a.L[D1].bias_off + c0 + i];
      store_row<BF16, TERMS>(sA, TSTRIDE, t, c0, W, v);
    }
    sync_for_mma();
    // mlp2 first layer: relu(hidden W^T + per-ray (bias + PE term))
    ok = __syncthreads_and(
        tc_layer<BF16, TERMS>(a.L[D1 + 1], sB, wterm, sA, TSTRIDE, tmem, bar, phase, DV_SAVE(D1 + 1)));
    if (!ok) break;
    {
      const int ray = valid ? __ldg(a.seg_ray + s) : 0;
      const float4* po = reinterpret_cast<const float4*>(a.pe_out + (long long)ray * W);
#pragma unroll
      for (int c0 = 0; c0 < W; c0 += EPI_COLS<TERMS>) {
        acc_row<TERMS>(trow + c0, a.L[D1 + 1].N, v);
#pragma unroll
        for (int i = 0; i < EPI_COLS<TERMS>; i += 4) {
          const float4 p = __ldg(po + (c0 + i) / 4);
          v[i] = fmaxf(v[i] + p.x, 0.f);
          v[i + 1] = fmaxf(v[i + 1] + p.y, 0.f);
          v[i + 2] = fmaxf(v[i + 2] + p.z, 0.f);
          v[i + 3] = fmaxf(v[i + 3] + p.w, 0.f);
        }
        store_row<BF16, TERMS>(sA, TSTRIDE, t, c0, W, v);
      }
    }
    sync_for_mma();
    // mlp2 output: 3 logits -> sigmoid
    ok = __syncthreads_and(
        tc_layer<BF16, TERMS>(a.L[D1 + 2], sB, wterm, sA, TSTRIDE, tmem, bar, phase, DV_SAVE(D1 + 2)));
#undef DV_SAVE
    if (!ok) break;
    {
      float o[4];
      acc_row4<TERMS>(trow, a.L[D1 + 2].N, o);
      const int bo = a.L[D1 + 2].bias_off;
      if (valid)
        a.out4[s] = make_float4(sigma, sigmoidf_acc(o[0] + sBias[bo]), sigmoidf_acc(o[1] + sBias[bo + 1]),
                                sigmoidf_acc(o[2] + sBias[bo + 2]));
    }
    tc::fence_before_sync();
    __syncthreads();  // the next gather overwrites A
  }
  if (!ok && t == 0 && a.err) atomicExch(a.err, 1);
  if (a.save != nullptr && t == 0) tc::bulk_wait_all();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tmem, NCOLS);
}

// The persistent grid holds as many CTAs per SM as registers, shared memory
// and TMEM (512 columns) allow together (the occupancy API under-reports
// kernels that allocate TMEM).
template <int C, int W, int D1, int BF16, int TERMS = 1>
int launch_decode_fwd_tc(const TcArgs& a, cudaStream_t st) {
  // split form: two column blocks of the widest N
  constexpr int NCOLS = TERMS > 1 ? (W == 32 ? 128 : 256) : (W == 32 ? 64 : 128);
  constexpr int KMAX = C > W ? C : W;
  const size_t smem = (size_t)TERMS * a.wbytes + (size_t)a.nbias * 4 + (size_t)TERMS * 128 * KMAX * 2 + 16;
  auto k = decode_fwd_tc<C, W, D1, BF16, NCOLS, TERMS>;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return DV_ERR_CUDA;
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
  const long long tiles = (a.S + 127) / 128;
  const long long grid = std::min<long long>(tiles, (long long)sms * res.per_sm);
  k<<<(unsigned)grid, 128, res.dyn_smem, st>>>(a);
  DV_TRY_LAUNCH();
  return DV_OK;
}

// Exercises the bounded completion wait that every tensor-core kernel uses
// (tc::mbar_wait_bounded): one wait on an mbarrier that nobody arrives on
// must give up after `limit` polls and report it; one after an arrival must
// succeed.  status[0] = 1 if the unarrived wait timed out, status[1] = 0 if
// the arrived wait completed.
__global__ void wait_selftest_kernel(uint32_t limit, int* status) {
  __shared__ __align__(8) uint64_t bar[2];
  tc::mbar_init(&bar[0], 1);
  tc::mbar_init(&bar[1], 1);
  tc::fence_mbar_init();
  status[0] = tc::mbar_wait_bounded(&bar[0], 0, limit) ? 0 : 1;
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_u32(&bar[1])) : "memory");
  status[1] = tc::mbar_wait_bounded(&bar[1], 0, limit) ? 0 : 1;
}

// Weight image gather for a refresh after an optimizer step: out term t, entry
// i = term t of ext[index[i]], where ext[0] = 0 and ext[j] = params[j - 1].
// form 0: FP32 (biases), 1: BF16, 2: FP16, 3: three BF16 terms, each the
// round-to-nearest-even of what the previous ones left (the residuals are
// exact in FP32), term t at out + t * n * 2 bytes.
__global__ void tc_image_kernel(const float* __restrict__ params, long long n_params,
                                const int64_t* __restrict__ index, long long n, int form, void* out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const long long j = index[i];
    const float x = (j > 0 && j <= n_params) ? params[j - 1] : 0.f;
    if (form == 0) {
      static_cast<float*>(out)[i] = x;
    } else if (form == 2) {
      static_cast<__half*>(out)[i] = __float2half_rn(x);
    } else {
      __nv_bfloat16* o = static_cast<__nv_bfloat16*>(out);
      float r = x;
      const int terms = form == 3 ? 3 : 1;
      for (int t = 0; t < terms; ++t) {
        const __nv_bfloat16 b = __float2bfloat16_rn(r);
        o[t * n + i] = b;
        r = __fsub_rn(r, __bfloat162float(b));
      }
    }
  }
}

}  // namespace dv

using namespace dv;

// Checks the arguments of a tensor-core forward launch and fills TcArgs;
// terms: operand terms (1, or 3 for the split-operand form; the save record
// then holds two terms of every layer input).
static int decode_fwd_tc_args(TcArgs& a, int kind, int channels, int terms, const void* wblob, int wbytes,
                              const float* bias, int nbias, const int* layers, int n_layers, const float* voxels,
                              const void* voxels16, int nvx, int nvy, int nvz, const float* seg, const int* seg_ray,
                              long long n_seg, const int64_t* n_seg_dev, const float* pe_out, float* out4, void* save,
                              long long save_capacity, int* err) {
  const int d1 = kind == 32 ? 2 : (kind == 64 ? 1 : -1);
  DV_CHECK(d1 > 0 && n_layers == d1 + 3 && n_layers <= TC_MAX_LAYERS, DV_ERR_ARG);
  DV_CHECK((kind == 32 && channels == 32) || (kind == 64 && (channels == 32 || channels == 64)), DV_ERR_UNSUPPORTED);
  DV_CHECK(wblob && bias && layers && voxels && seg && seg_ray && pe_out && out4, DV_ERR_ARG);
  DV_CHECK(wbytes > 0 && wbytes % 16 == 0 && nbias > 0 && nbias % 4 == 0, DV_ERR_ARG);
  DV_CHECK(((uintptr_t)wblob & 15) == 0 && ((uintptr_t)voxels & 15) == 0 && ((uintptr_t)out4 & 15) == 0, DV_ERR_ARG);
  DV_CHECK(voxels16 == nullptr || ((uintptr_t)voxels16 & 15) == 0, DV_ERR_ARG);
  a.grid = voxels;
  a.grid16 = reinterpret_cast<const uint16_t*>(voxels16);
  a.nvx = nvx;
  a.nvy = nvy;
  a.nvz = nvz;
  a.seg = seg;
  a.seg_ray = seg_ray;
  a.S = n_seg;
  a.S_dev = n_seg_dev;
  a.pe_out = pe_out;
  a.out4 = reinterpret_cast<float4*>(out4);
  a.wblob = reinterpret_cast<const uint8_t*>(wblob);
  a.wbytes = wbytes;
  a.bias = bias;
  a.nbias = nbias;
  a.err = err;
  const int W = kind;
  for (int l = 0; l < n_layers; ++l) {
    a.L[l].b_off = layers[4 * l];
    a.L[l].K = layers[4 * l + 1];
    a.L[l].N = layers[4 * l + 2];
    a.L[l].bias_off = layers[4 * l + 3];
    const TcLayer& L = a.L[l];
    // every operand must lie inside the blob, on a 16-byte boundary, with legal MMA shapes
    DV_CHECK(L.K % 16 == 0 && L.N % 16 == 0 && L.N >= 16 && L.N <= 256 && L.b_off % 16 == 0, DV_ERR_ARG);
    DV_CHECK((long long)L.b_off + (long long)L.N * L.K * 2 <= wbytes && L.bias_off + L.N <= nbias, DV_ERR_ARG);
    DV_CHECK(L.N <= (W == 32 ? 64 : 128), DV_ERR_ARG);
  }
  // the split form's images regrouped in shared memory, layer by layer
  {
    long long off = 0;
    for (int l = 0; l < n_layers; ++l) {
      a.L[l].s_off = (int)off;
      off += 3LL * a.L[l].N * a.L[l].K * 2;
    }
    DV_CHECK(terms == 1 || off <= 3LL * wbytes, DV_ERR_ARG);
  }
  // saved layer inputs: one record of sum(256 K) bytes (per saved term) per 128-segment tile
  if (save != nullptr) {
    const int saved_terms = terms > 1 ? 2 : 1;
    int off = 0;
    for (int l = 0; l < n_layers; ++l) {
      a.save_off[l] = off;
      off += 256 * a.L[l].K * saved_terms;
    }
    a.save = reinterpret_cast<uint8_t*>(save);
    a.save_bytes = off;
    DV_CHECK(((uintptr_t)save & 15) == 0, DV_ERR_ARG);
    DV_CHECK((n_seg + 127) / 128 * (long long)off <= save_capacity, DV_ERR_ARG);
  }
  // layer shapes the kernel assumes
  DV_CHECK(a.L[0].K == channels && a.L[0].N == W, DV_ERR_ARG);
  for (int l = 1; l < d1; ++l) DV_CHECK(a.L[l].K == W && a.L[l].N == W, DV_ERR_ARG);
  DV_CHECK(a.L[d1].K == W && a.L[d1].N >= W + 4, DV_ERR_ARG);
  DV_CHECK(a.L[d1 + 1].K == W && a.L[d1 + 1].N == W && a.L[d1 + 2].K == W && a.L[d1 + 2].N >= 16, DV_ERR_ARG);
  return DV_OK;
}

extern "C" {

int dv_decode_fwd_tc(int kind, int channels, int bf16, const void* wblob, int wbytes, const float* bias, int nbias,
                     const int* layers, int n_layers, const float* voxels, const void* voxels16, int nvx, int nvy,
                     int nvz, const float* seg, const int* seg_ray, long long n_seg, const int64_t* n_seg_dev,
                     const float* pe_out, float* out4, void* save, long long save_capacity, int* err,
                     void* stream) {
  DV_CHECK(n_seg >= 0 && (bf16 == 0 || bf16 == 1), DV_ERR_ARG);
  if (n_seg == 0) return DV_OK;
  TcArgs a{};
  const int rc = decode_fwd_tc_args(a, kind, channels, 1, wblob, wbytes, bias, nbias, layers, n_layers, voxels,
                                    voxels16, nvx, nvy, nvz, seg, seg_ray, n_seg, n_seg_dev, pe_out, out4, save,
                                    save_capacity, err);
  if (rc != DV_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  if (kind == 32) return bf16 ? launch_decode_fwd_tc<32, 32, 2, 1>(a, st) : launch_decode_fwd_tc<32, 32, 2, 0>(a, st);
  if (channels == 32)
    return bf16 ? launch_decode_fwd_tc<32, 64, 1, 1>(a, st) : launch_decode_fwd_tc<32, 64, 1, 0>(a, st);
  return bf16 ? launch_decode_fwd_tc<64, 64, 1, 1>(a, st) : launch_decode_fwd_tc<64, 64, 1, 0>(a, st);
}

int dv_decode_fwd_tc_split(int kind, int channels, const void* wblob, int wbytes, const float* bias, int nbias,
                           const int* layers, int n_layers, const float* voxels, int nvx, int nvy, int nvz,
                           const float* seg, const int* seg_ray, long long n_seg, const int64_t* n_seg_dev,
                           const float* pe_out, float* out4, void* save, long long save_capacity, int* err,
                           void* stream) {
  DV_CHECK(n_seg >= 0, DV_ERR_ARG);
  if (n_seg == 0) return DV_OK;
  TcArgs a{};
  const int rc = decode_fwd_tc_args(a, kind, channels, 3, wblob, wbytes, bias, nbias, layers, n_layers, voxels,
                                    nullptr, nvx, nvy, nvz, seg, seg_ray, n_seg, n_seg_dev, pe_out, out4, save,
                                    save_capacity, err);
  if (rc != DV_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  if (kind == 32) return launch_decode_fwd_tc<32, 32, 2, 1, 3>(a, st);
  if (channels == 32) return launch_decode_fwd_tc<32, 64, 1, 1, 3>(a, st);
  return launch_decode_fwd_tc<64, 64, 1, 1, 3>(a, st);
}

long long dv_decode_tc_split_save_bytes(int kind, int channels, long long n_seg) {
  const int d1 = kind == 32 ? 2 : (kind == 64 ? 1 : -1);
  if (d1 < 0 || n_seg < 0) return -1;
  const long long record = 2 * 256LL * (channels + (d1 + 2) * kind);
  return (n_seg + 127) / 128 * record;
}

int dv_wait_selftest(int limit, int* status, void* stream) {
  DV_CHECK(limit > 0 && limit <= (1 << 20) && status, DV_ERR_ARG);
  wait_selftest_kernel<<<1, 1, 0, (cudaStream_t)stream>>>((uint32_t)limit, status);
  DV_TRY_LAUNCH();
  return DV_OK;
}

long long dv_decode_tc_save_bytes(int kind, int channels, long long n_seg) {
  const int d1 = kind == 32 ? 2 : (kind == 64 ? 1 : -1);
  if (d1 < 0 || n_seg < 0) return -1;
  const long long record = 256LL * (channels + (d1 + 2) * kind);
  return (n_seg + 127) / 128 * record;
}

int dv_tc_image(const float* params, long long n_params, const int64_t* index, long long n, int form, void* out,
                void* stream) {
  DV_CHECK(n >= 0 && n_params >= 0 && form >= 0 && form <= 3, DV_ERR_ARG);
  if (n == 0) return DV_OK;
  DV_CHECK(index && out && (params || n_params == 0), DV_ERR_ARG);
  const unsigned blocks = (unsigned)std::min<long long>((n + 255) / 256, 4LL * 152);
  tc_image_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(params, n_params, index, n, form, out);
  DV_TRY_LAUNCH();
  return DV_OK;
}

}  // extern "C"
