// Tensor-core (tcgen05) backward of the DIVeR32 decoder with split BF16
// operands: FP32-grade gradients from BF16 tensor cores.
//
// Every FP32 operand is carried as a sum of BF16 terms (tc::split_pair):
//   - delta propagation  dL/d input = delta @ W: delta and W as three terms
//     each, the six products whose term indices add up to at most 2;
//   - weight gradient    dW += delta^T @ activation: two terms each, all four
//     products (FP32 accumulators resident in TMEM for the CTA's life);
//   - bias gradient      dB += delta^T @ ones: the column sums of the two-term
//     delta, also accumulated in TMEM (layer 3's from a column of ones in the
//     PE tile, which the weight-gradient MMA already reads).
// Products are accumulated in FP32 in TMEM, so the propagated deltas and the
// gradients keep about 2^-24 (propagation) and 2^-16 (weight gradients) of
// relative precision per product; emulating the kernel's arithmetic on the
// CPU gives gradients within a few 1e-7 (grid) and 1e-6 (weights) relative
// of an FP64 backward, where a single BF16 term gives 1e-2.
//
// A tcgen05.mma costs the tensor core about 46 clocks whatever its shape up
// to N = 64 (M = 64 or 128, K = 16), so the layout is chosen for few, wide
// MMAs:
//   - the delta tile is one [128][3 x 48] tile, term i in columns 48i..48i+47;
//     read transposed with M = 128 it puts delta terms 0 and 1 in accumulator
//     rows 0..47 and 48..95 of ONE MMA (rows 96..127 see term 2 and are never
//     read);
//   - the saved activations and the PE tile are [128][2 x 32] tiles, term j
//     in columns 32j..32j+31, so one MMA of N = 64 takes both terms;
//   - the propagation images sit layer by layer with the three weight terms
//     side by side along N: per 16 columns of K, delta_0 x [W0|W1] and
//     delta_1 x [W0|W1] (N = 64), delta_0 x W2 into columns 32..63 and
//     delta_2 x W0 into columns 0..31; the epilogue adds the two column blocks.
// Per 128-segment tile that is 40 propagation, 48 weight-gradient and 32
// bias-gradient MMAs.
//
// The forward is not recomputed: dv_decode_fwd_tc_split saved, per tile of 128
// segments, every layer's input as a [128][2 x 32] two-term tile (X0, A1, A2,
// hidden, A4; 16 KiB each), and its FP32 out4 gives the colour logits'
// sigmoid.  The record is read into shared memory by bulk async copies, one
// per layer slot.
//
// One CTA per SM, 288 threads: chain thread t < 256 owns segment row
// r = t % 128 (TMEM lane r; warps w and w + 4 share a lane quadrant) and half
// h = t / 128 of each row's columns in the epilogues; lane 0 of warp 8 issues
// the MMAs and the record loads.  The scatter of a tile's feature gradient
// into the grid runs on the chain threads while the next tile's MMAs run.
// Shared memory (about 184 KiB): the propagation images, the saved record in
// five per-layer slots, the PE tile, the delta tile, a tile of ones and the
// FP32 staging rows of the feature gradient.  TMEM: all 512 columns (64
// working, 384 weight-gradient and 64 bias-gradient columns).
// Reference semantics: the autograd backward of model/diver.py:159-180.
#include "common.cuh"
#include "integrate.cuh"
#include "mlp.cuh"
#include "tc.cuh"

#include <algorithm>

namespace dv {
namespace bws {

constexpr int C = 32, W = 32;
constexpr int NL = 5;
constexpr int CHAIN = 256;             // the layer chain's threads: two per segment row (warps 0-7)
constexpr int ISSUER = CHAIN;          // lane 0 of warp 8: issues the MMAs and the record loads
constexpr int THREADS = CHAIN + 32;
constexpr int FD = 48;              // delta columns per term (K of the widest propagation MMA)
constexpr int DW = 3 * FD;          // delta tile columns: the three terms side by side
constexpr int TILE = 128 * 32 * 2;  // one term of a [128][32] BF16 tile
constexpr int DTILE = 128 * FD * 2; // one term's share of the delta tile
constexpr int TMEM_COLS = 512;      // 64 working + 384 weight-gradient + 64 bias-gradient columns
// layer: 0 (C->W), 1 (W->W), 2 (W->W+1: sigma, hidden), 3 (W+27->W), 4 (W->3)
__host__ __device__ constexpr int IN(int l) { return l == 0 ? C : (l == 3 ? W + PE_DIM : W); }
__host__ __device__ constexpr int OUT(int l) { return l == 2 ? W + 1 : (l == 4 ? 3 : W); }
__host__ __device__ constexpr int OUT4(int l) { return pad4(OUT(l)); }
__host__ __device__ constexpr int NBLK(int l) { return l == 3 ? 2 : 1; }  // 32-column input blocks (layer 3: + PE)
// weight gradient of layer l: per input block, 64 columns (activation terms 0 and 1)
__host__ __device__ constexpr int DWCOL(int l) { return l == 0 ? 64 : DWCOL(l - 1) + 64 * NBLK(l - 1); }
// bias gradient of layer l != 3 (column 0 of 16); layer 3's is column 27 of its PE block
__host__ __device__ constexpr int DBCOL(int l) { return 448 + 16 * (l < 3 ? l : l - 1); }
constexpr int PE_ONES = 27;  // the PE tile's column of ones (PE_DIM = 27 values before it)
__host__ __device__ constexpr int KPROP(int l) { return l == 4 ? 16 : (l == 2 ? W + 16 : W); }  // propagation K
// propagation image of layer l in shared memory: [3 terms x 32 rows][KPROP(l)],
// the three terms side by side along N, layers one after the other
__host__ __device__ constexpr int PIMG(int l) { return 32 * KPROP(l) * 2; }  // one term's bytes
__host__ __device__ constexpr int POFF(int l) { return l == 0 ? 0 : POFF(l - 1) + 3 * PIMG(l - 1); }
constexpr uint32_t RECORD = 5 * 2 * TILE;  // saved record of one tile: 5 layer inputs, [128][2 x 32] each
constexpr uint32_t ONES_BYTES = 128 * 16 * 2;  // a [128][16] BF16 tile of ones

struct Args {
  int nvx, nvy, nvz;
  const float* seg;
  const int* seg_ray;
  long long S;           // segment count, or capacity when S_dev is set
  const int64_t* S_dev;  // optional device-held count (clamped to S)
  const float* pe_feat;  // [B][28]
  const float4* d4;      // [S] (dL/dsigma, dL/drgb)
  const float4* out4;    // [S] (sigma, sigmoid rgb) of the forward
  const uint8_t* saved;  // RECORD bytes per tile
  float* grad_grid;
  float* grad_params;    // packed torch layout
  uint8_t* touched;      // optional: a byte per grid row, set at each segment's lower corner
  int w_off[NL], b_off[NL];
  const uint8_t* wb;     // transposed weight images, three terms of wterm bytes
  int wterm;
  int b_img[NL];         // byte offset of layer l's image inside a term
  int* err;
};

// Shared-memory layout (byte offsets; the propagation images take 3 x 10240 bytes).
struct Layout {
  uint32_t bb, rec, pe, d, ones, stage, bar;
  __host__ __device__ static Layout make() {
    Layout L;
    L.bb = 0;
    L.rec = (uint32_t)(POFF(NL) + 1023) / 1024 * 1024;
    L.pe = L.rec + RECORD;
    L.d = L.pe + 2 * TILE;
    L.ones = L.d + 3 * DTILE;
    L.stage = L.ones + ONES_BYTES;
    L.bar = L.stage + 128 * (C + 4) * 4;
    return L;
  }
  // barriers: MMA completion, NL record slots; then the TMEM address and the abort flag
  __host__ __device__ uint32_t bytes() const { return bar + 8 * (1 + NL) + 16; }
};

// Writes n values (multiple of 8) of row r, columns c0.., as three BF16 terms
// into the delta tile (term i in columns FD * i + c).
__device__ __forceinline__ void put3(uint8_t* D, int r, int c0, const float* v, int n) {
#pragma unroll
  for (int c = 0; c < n; c += 8) {
    uint32_t x[3], y[3], z[3], u[3];
    tc::split_pair<3>(v[c], v[c + 1], x);
    tc::split_pair<3>(v[c + 2], v[c + 3], y);
    tc::split_pair<3>(v[c + 4], v[c + 5], z);
    tc::split_pair<3>(v[c + 6], v[c + 7], u);
#pragma unroll
    for (int i = 0; i < 3; ++i)
      *reinterpret_cast<uint4*>(D + tc::kmajor_offset(r, FD * i + c0 + c, DW)) = make_uint4(x[i], y[i], z[i], u[i]);
  }
}

// Same with two terms into a [128][2 x 32] tile (term j in columns 32 j + c).
__device__ __forceinline__ void put2(uint8_t* tile, int r, int c0, const float* v, int n) {
#pragma unroll
  for (int c = 0; c < n; c += 8) {
    uint32_t x[2], y[2], z[2], u[2];
    tc::split_pair<2>(v[c], v[c + 1], x);
    tc::split_pair<2>(v[c + 2], v[c + 3], y);
    tc::split_pair<2>(v[c + 4], v[c + 5], z);
    tc::split_pair<2>(v[c + 6], v[c + 7], u);
#pragma unroll
    for (int j = 0; j < 2; ++j)
      *reinterpret_cast<uint4*>(tile + tc::kmajor_offset(r, 32 * j + c0 + c, 64)) = make_uint4(x[j], y[j], z[j], u[j]);
  }
}

// Zeroes v[i] where the activation (leading term of a [128][2 x 32] record
// tile, row r, columns c0..c0+n-1) is not positive: the ReLU derivative.  The
// leading BF16 term has the sign of the FP32 activation (and is zero only with it).
__device__ __forceinline__ void relu_mask(const uint8_t* tile, int r, int c0, float* v, int n) {
#pragma unroll
  for (int c = 0; c < n; c += 8) {
    const uint4 w = *reinterpret_cast<const uint4*>(tile + tc::kmajor_offset(r, c0 + c, 64));
    const uint32_t x[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (!(tc::bf_lo(x[j]) > 0.f)) v[c + 2 * j] = 0.f;
      if (!(tc::bf_hi(x[j]) > 0.f)) v[c + 2 * j + 1] = 0.f;
    }
  }
}

// Propagation: TMEM columns [0, 32) + [32, 64) = delta [128][K] x W^T, for
// delta three terms of the delta tile (term i starting at column FD i) and
// the layer's image [3 x 32][K] (weight term j in rows 32j..32j+31): per 16
// columns of K, delta_0 x [W0|W1] and delta_1 x [W0|W1] into columns 0..63,
// delta_0 x W2 into 32..63 and delta_2 x W0 into 0..31.
__device__ __forceinline__ void mma_prop(uint32_t tmem, const uint8_t* D, const uint8_t* img, int K) {
  constexpr uint32_t sboA = (DW / 8) * 128, term = (FD / 8) * 128;
  const uint64_t a0 = tc::smem_desc(tc::smem_u32(D), 128, sboA);
  const uint64_t b0 = tc::smem_desc(tc::smem_u32(img), 128, (uint32_t)(K / 8) * 128);
  const uint32_t i64 = tc::idesc_f16(128, 64, 1), i32 = tc::idesc_f16(128, 32, 1);
#pragma unroll
  for (int k = 0; k < K / 16; ++k) {
    const uint64_t ak = tc::desc_plus(a0, k * 256), bk = tc::desc_plus(b0, k * 256);
    tc::mma_f16(tmem, ak, bk, i64, k > 0 ? 1u : 0u);
    tc::mma_f16(tmem, tc::desc_plus(ak, term), bk, i64, 1u);
    tc::mma_f16(tmem + 32, ak, tc::desc_plus(bk, 2 * 32 * K * 2), i32, 1u);
    tc::mma_f16(tmem, tc::desc_plus(ak, 2 * term), bk, i32, 1u);
  }
}

// Transposed view of the delta tile as the A operand of the gradient MMAs:
// M = 128 rows = delta tile columns 0..127 (terms 0 and 1 in rows 0..47 and
// 48..95), K = 16 segments per MMA.
__device__ __forceinline__ uint64_t delta_t_desc(const uint8_t* D) {
  constexpr uint32_t lbo = (DW / 8) * 128;  // next 8 segments
  return tc::smem_desc(tc::smem_u32(D), lbo, 128);
}
constexpr uint32_t DELTA_T_K = 2 * (DW / 8) * 128;  // bytes per 16 segments of that view

// Weight gradient over the tile's 128 segments: TMEM dW[128][64] +=
// delta^T x act, act a [128][2 x 32] tile read transposed (N = 64: both terms).
__device__ __forceinline__ void mma_dw(uint32_t tmem, const uint8_t* D, const uint8_t* act, bool accumulate) {
  const uint32_t idesc = tc::idesc_f16(128, 64, 1) | (1u << 15) | (1u << 16);
  constexpr uint32_t lboB = (64 / 8) * 128;
  const uint64_t a0 = delta_t_desc(D), b0 = tc::smem_desc(tc::smem_u32(act), lboB, 128);
#pragma unroll
  for (int k = 0; k < 8; ++k)
    tc::mma_f16(tmem, tc::desc_plus(a0, k * DELTA_T_K), tc::desc_plus(b0, k * 2 * lboB), idesc,
                (accumulate || k > 0) ? 1u : 0u);
}

// Bias gradient over the tile's 128 segments: TMEM dB[128][16] += delta^T x
// ones, every column the column sum of the delta (terms 0 and 1 in rows 0..47
// and 48..95; the ones are exact in BF16 and any reading of the all-ones tile
// is the same).
__device__ __forceinline__ void mma_db(uint32_t tmem, const uint8_t* D, const uint8_t* ones, bool accumulate) {
  const uint32_t idesc = tc::idesc_f16(128, 16, 1) | (1u << 15) | (1u << 16);
  constexpr uint32_t lboB = (16 / 8) * 128;
  const uint64_t a0 = delta_t_desc(D), b0 = tc::smem_desc(tc::smem_u32(ones), lboB, 128);
#pragma unroll
  for (int k = 0; k < 8; ++k)
    tc::mma_f16(tmem, tc::desc_plus(a0, k * DELTA_T_K), tc::desc_plus(b0, k * 2 * lboB), idesc,
                (accumulate || k > 0) ? 1u : 0u);
}

// Scatter of a finished tile's feature gradient (FP32 staging rows) into the
// corner rows of its segments, spread over the next tile's first HRUN layer
// steps, where it fills the wait for their MMAs: thread t takes channel quad
// q = t % 8 of the HRUN consecutive segments HRUN * (t / 8).. (a half-run),
// one segment per step.  Consecutive segments of a ray usually sit in
// face-adjacent voxels and share four corner rows: the shared corners'
// contributions are added in registers and reach memory with one atomic
// instead of two.  A merge needs both voxels whole (upper corners not
// clamped) and one unit step along one axis, so the merged rows are the same
// rows.  Threads q and q + 4 of a half-run load segment q % 4's coordinates;
// the others take them by shuffles.
constexpr int HRUN = 4;
static_assert((C / 4) * (128 / HRUN) == CHAIN, "one thread per (channel quad, half-run)");

struct Scatter {
  long long s0 = -1;  // first segment of this thread's half-run; -1: nothing to scatter
  int ls0 = 0, q = 0;
  float crd[6];       // coordinates of segment s0 + q % HRUN
  float4 pend[8];     // contributions of the previous segment's corners not yet in memory
  SegCorner prev{};
  bool have = false, prev_whole = false;

  __device__ __forceinline__ void start(const Args& a, long long tile, int t, long long S) {
    q = t % (C / 4);
    ls0 = (t / (C / 4)) * HRUN;
    s0 = tile * 128 + ls0;
    const long long s = s0 + q % HRUN;
#pragma unroll
    for (int i = 0; i < 6; ++i) crd[i] = s < S ? __ldg(a.seg + s * 6 + i) : 0.f;
    have = false;
  }

  // Segment k of the half-run (every lane takes every shuffle); k = HRUN - 1
  // also writes what is still pending and ends the scatter.
  __device__ __forceinline__ void step(const Args& a, const float* stage, int k, long long S) {
    float p[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) p[i] = __shfl_sync(0xffffffffu, crd[i], k, C / 4);
    if (s0 + k < S) {
      const SegCorner sc = segment_corners(p[0], p[1], p[2], p[3], p[4], p[5], a.nvx, a.nvy, a.nvz);
      // the row marks for the next step's sparse clear (dv_mark_corner_rows' rule)
      if (a.touched && q == 0) a.touched[((long long)sc.z * a.nvy + sc.y) * a.nvx + sc.x] = 1;
      const float4 g = *reinterpret_cast<const float4*>(stage + (ls0 + k) * (C + 4) + 4 * q);
      const bool whole = sc.x1 == sc.x + 1 && sc.y1 == sc.y + 1 && sc.z1 == sc.z + 1;
      int axis = -1;
      bool up = false;
      if (have && whole && prev_whole) {
        const int dx = sc.x - prev.x, dy = sc.y - prev.y, dz = sc.z - prev.z;
        if (abs(dx) + abs(dy) + abs(dz) == 1) {
          axis = dx != 0 ? 0 : (dy != 0 ? 1 : 2);
          up = dx + dy + dz > 0;
        }
      }
      // the previous segment's corners off the shared face go to memory
      if (have) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const bool shared = axis >= 0 && ((j >> axis) & 1) == (up ? 1 : 0);
          if (!shared) red_add4(a.grad_grid + corner_row(prev, j, a.nvx, a.nvy) * C + 4 * q, pend[j]);
        }
      }
      float4 nx[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const float w = sc.w[j];
        float4 c = make_float4(w * g.x, w * g.y, w * g.z, w * g.w);
        if (axis >= 0 && ((j >> axis) & 1) == (up ? 0 : 1)) {
          const float4 o = axis == 0 ? pend[j ^ 1] : (axis == 1 ? pend[j ^ 2] : pend[j ^ 4]);
          c.x += o.x;
          c.y += o.y;
          c.z += o.z;
          c.w += o.w;
        }
        nx[j] = c;
      }
#pragma unroll
      for (int j = 0; j < 8; ++j) pend[j] = nx[j];
      prev = sc;
      prev_whole = whole;
      have = true;
    }
    if (k == HRUN - 1) {
      if (have) {
#pragma unroll
        for (int j = 0; j < 8; ++j) red_add4(a.grad_grid + corner_row(prev, j, a.nvx, a.nvy) * C + 4 * q, pend[j]);
      }
      have = false;
      s0 = -1;
    }
  }
};

// Named barrier of the chain (barrier 0 is __syncthreads).
constexpr int BAR_CHAIN = 1;

__device__ __forceinline__ void named_sync(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }
// AND of `v` over the n threads of named barrier `id` (all of them wait).
__device__ __forceinline__ bool named_and(int id, int n, bool v) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 q, %1, 0;\n bar.red.and.pred p, %2, %3, q;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(r)
      : "r"((uint32_t)v), "r"(id), "r"(n)
      : "memory");
  return r != 0;
}

// Chain-group barrier that also orders generic-proxy shared-memory writes
// before the tensor core's reads (and tcgen05 work across the barrier).
__device__ __forceinline__ void chain_sync() {
  tc::fence_before_sync();
  tc::fence_async_smem();
  named_sync(BAR_CHAIN, THREADS);
}

// PE tile row r, columns 16h..16h+15 (PE_DIM = 27 values, then a one in
// column PE_ONES for layer 3's bias gradient, zeros after), two terms.
__device__ __forceinline__ void write_pe(const Args& a, uint8_t* PE, int ray, int r, int h) {
  float v[16];
  const float* pf = a.pe_feat + (long long)ray * PE_PAD + 16 * h;
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = (16 * h + i < PE_DIM) ? __ldg(pf + i) : (16 * h + i == PE_ONES ? 1.f : 0.f);
  put2(PE, r, 16 * h, v, 16);
}

// Delta of the colour logits (dL/drgb * sigmoid') into columns 0..15 of row r.
__device__ __forceinline__ void write_delta4(uint8_t* D, int r, float4 g, float4 oc) {
  float v[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = 0.f;
  v[0] = g.y * oc.y * (1.f - oc.y);
  v[1] = g.z * oc.z * (1.f - oc.z);
  v[2] = g.w * oc.w * (1.f - oc.w);
  put3(D, r, 0, v, 16);
}

// This thread's row of the propagation result, columns c..c+15 (taddr =
// lane base + c): the two column blocks of mma_prop added.
__device__ __forceinline__ void prop_row16(uint32_t taddr, float* v) {
  float b[16];
  tc::ld_32x32b_x16(taddr, v);
  tc::ld_32x32b_x16(taddr + 32, b);
  tc::ld_wait();
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] += b[i];
}

// Same for columns 0..31.
__device__ __forceinline__ void prop_row32(uint32_t taddr, float* v) {
  prop_row16(taddr, v);
  prop_row16(taddr + 16, v + 16);
}

// One tile per step of the persistent loop: the five layer steps, each the
// propagation and gradient MMAs and the epilogue that forms the next delta;
// the last stages the tile's feature gradient (FP32), which the next tile's
// first four steps scatter into the grid (Scatter) while their MMAs run.
// The saved record sits in five per-layer slots, each with its own mbarrier:
// when a layer step of tile i is done with its slot, that slot is refilled
// with tile i + gridDim.x's layer input, so the next tile's loads run behind
// the rest of this tile.  The PE tile and the first delta of the next tile are
// also written as soon as this tile is done with them.
__global__ void __launch_bounds__(THREADS, 1) decode_bwd_tc_split_kernel(const Args a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  const Layout lay = Layout::make();
  uint8_t* Bb = smem + lay.bb;
  uint8_t* REC = smem + lay.rec;
  uint8_t* PE = smem + lay.pe;
  uint8_t* D = smem + lay.d;
  uint8_t* ONES = smem + lay.ones;
  float* stage = reinterpret_cast<float*>(smem + lay.stage);  // [128][C + 4] FP32
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + lay.bar);
  uint64_t* bar_rec = bar + 1;  // [NL]: completion of slot l's record load
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 1 + NL);

  const int t = threadIdx.x, warp = t >> 5;
  const bool chain = t < CHAIN, issuer = t == ISSUER;
  const int r = t & 127, h = (t >> 7) & 1;
  const long long S = segment_total(a.S, a.S_dev);
  const long long tiles = (S + 127) / 128;

  // propagation images, regrouped layer by layer with the three terms side by side
#pragma unroll
  for (int l = 0; l < NL; ++l)
    for (int i = t; i < 3 * PIMG(l) / 16; i += THREADS) {
      const int j = i / (PIMG(l) / 16), o = i % (PIMG(l) / 16);
      reinterpret_cast<uint4*>(Bb + POFF(l))[i] =
          __ldg(reinterpret_cast<const uint4*>(a.wb + j * a.wterm + a.b_img[l]) + o);
    }
  for (int i = t; i < 3 * DTILE / 16; i += THREADS) reinterpret_cast<uint4*>(D)[i] = make_uint4(0, 0, 0, 0);
  for (int i = t; i < (int)ONES_BYTES / 16; i += THREADS)
    reinterpret_cast<uint4*>(ONES)[i] = make_uint4(0x3f803f80u, 0x3f803f80u, 0x3f803f80u, 0x3f803f80u);  // bf16 1.0
  if (t == 0) {
    tc::mbar_init(bar, 1);
    for (int l = 0; l < NL; ++l) tc::mbar_init(bar_rec + l, 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(tslot, TMEM_COLS);
    tc::tmem_relinquish();
  }
  tc::fence_before_sync();
  tc::fence_async_smem();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;

  {
    const uint32_t lane = (uint32_t)((warp & 3) * 32) << 16;
    const uint32_t trow = tmem + lane;
    uint32_t phase = 0, phase_rec = 0;  // phase_rec: bit l = parity of slot l's next completion
    uint32_t pending = 0;               // issuer: slots with a load in flight
    bool mma_inflight = false;          // issuer: an MMA batch committed and not yet waited for
    bool ok = true, first = true;
    float v[32];
    Scatter sc;  // the previous tile's feature-gradient scatter
    // the CTA's first tile: record loads, PE tile, first delta
    long long tile = blockIdx.x;
    if (tile < tiles) {
      if (issuer) {
        const uint8_t* rec = a.saved + tile * (long long)RECORD;
        for (int l = 0; l < NL; ++l) {
          tc::mbar_arrive_expect_tx(bar_rec + l, 2 * TILE);
          tc::bulk_load(REC + l * 2 * TILE, rec + l * 2 * TILE, 2 * TILE, bar_rec + l);
        }
        pending = (1u << NL) - 1;
      }
      const long long s = tile * 128 + r;
      const bool valid = s < S;
      if (chain) {
        write_pe(a, PE, valid ? __ldg(a.seg_ray + s) : 0, r, h);
        if (h == 0)
          write_delta4(D, r, valid ? a.d4[s] : make_float4(0.f, 0.f, 0.f, 0.f),
                       valid ? a.out4[s] : make_float4(0.f, 0.f, 0.f, 0.f));
      }
    }
    for (; tile < tiles && ok; tile += gridDim.x) {
      const long long s = tile * 128 + r;
      const bool valid = s < S;
      const long long next = tile + gridDim.x;
      const long long sn = next * 128 + r;
      const bool valid_next = next < tiles && sn < S;
      const float gx = chain && valid ? a.d4[s].x : 0.f;  // dL/dsigma of this row (layer 2's delta)
      chain_sync();  // the PE tile and the first delta are in place
      // layers last to first (unrolled: every layer constant is a compile-time value)
#pragma unroll
      for (int l = NL - 1; l >= 0; --l) {
        const uint8_t* act = REC + l * 2 * TILE;  // this layer's input, two terms TILE apart
        // this layer's record slot has arrived (bounded wait; the parities
        // advance only on success: after a timeout the abort path waits with them)
        const bool arrived = tc::mbar_wait_bounded(bar_rec + l, (phase_rec >> l) & 1u);
        if (arrived) phase_rec ^= 1u << l;
        if (issuer && arrived) {
          pending &= ~(1u << l);
          tc::fence_after_sync();
          mma_prop(tmem, D, Bb + POFF(l), KPROP(l));
          mma_dw(tmem + DWCOL(l), D, act, !first);
          if (l == 3)
            mma_dw(tmem + DWCOL(3) + 64, D, PE, !first);  // with layer 3's bias gradient (the ones column)
          else
            mma_db(tmem + DBCOL(l), D, ONES, !first);
          tc::mma_commit(bar);
          mma_inflight = true;
        }
        // while the MMAs run: one segment of the previous tile's scatter (steps 4..1)
        if (chain && l >= NL - HRUN && !first) sc.step(a, stage, NL - 1 - l, S);
        // if the issuer's slot wait gave up it issued nothing: every thread's MMA wait then
        // runs out too, and the AND below stops them all
        bool done = false;
        if (arrived) {
          done = tc::mbar_wait_bounded(bar, phase);
          if (done) {
            phase ^= 1u;
            if (issuer) mma_inflight = false;
          }
        }
        tc::fence_after_sync();
        ok = named_and(BAR_CHAIN, THREADS, arrived && done);
        if (!ok) break;
        if (!chain) {
          // the issuer warp has no rows
        } else if (l == 3) {
          // delta of layer 2: (dL/dsigma, d hidden[0..31]) in columns 0..32, zeros to 47;
          // half 0 writes columns 0..23, half 1 columns 24..47
          prop_row32(trow, v);
          float w[24];
          if (h == 0) {
            w[0] = gx;
#pragma unroll
            for (int i = 1; i < 24; ++i) w[i] = v[i - 1];
          } else {
#pragma unroll
            for (int i = 0; i < 24; ++i) w[i] = (i + 23 < W) ? v[i + 23] : 0.f;
          }
          put3(D, r, 24 * h, w, 24);
          // this tile's PE is consumed: the next tile's goes in now
          if (next < tiles) write_pe(a, PE, valid_next ? __ldg(a.seg_ray + sn) : 0, r, h);
        } else if (l > 0) {
          prop_row16(trow + 16 * h, v);
          relu_mask(act, r, 16 * h, v, 16);  // this layer's input is relu of the previous layer's output
          put3(D, r, 16 * h, v, 16);
        } else {
          // dL/dfeature (FP32) to the staging rows (the previous tile's scatter
          // finished in step 1), scattered during the next tile's steps
          float4 gn = make_float4(0.f, 0.f, 0.f, 0.f), on = gn;
          if (valid_next && h == 0) {
            gn = a.d4[sn];
            on = a.out4[sn];
          }
          prop_row16(trow + 16 * h, v);
          float* st = stage + r * (C + 4) + 16 * h;
#pragma unroll
          for (int i = 0; i < 16; i += 4)
            *reinterpret_cast<float4*>(st + i) =
                valid ? make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]) : make_float4(0.f, 0.f, 0.f, 0.f);
          sc.start(a, tile, t, S);
          // this tile's deltas are consumed: the next tile's first delta goes in now
          if (next < tiles && h == 0) write_delta4(D, r, gn, on);
        }
        chain_sync();  // D is complete for the next layer; every read of this layer's slot is done
        if (issuer && next < tiles) {
          // refill this layer's slot with the next tile's input
          tc::mbar_arrive_expect_tx(bar_rec + l, 2 * TILE);
          tc::bulk_load(REC + l * 2 * TILE, a.saved + next * (long long)RECORD + l * 2 * TILE, 2 * TILE,
                        bar_rec + l);
          pending |= 1u << l;
        }
      }
      if (!ok) break;
      first = false;
    }
    // the last tile's scatter (its staging rows are complete: every step ends with chain_sync)
    if (chain && ok && !first) {
#pragma unroll 1
      for (int k = 0; k < HRUN; ++k) sc.step(a, stage, k, S);
    }
    if (!ok) {
      if (issuer) {
        if (a.err) atomicExch(a.err, 1);
        // record loads and MMAs still in flight complete before the CTA frees
        // its shared memory and TMEM (bounded waits)
        for (int l = 0; l < NL; ++l)
          if ((pending >> l) & 1u) tc::mbar_wait_bounded(bar_rec + l, (phase_rec >> l) & 1u);
        if (mma_inflight) tc::mbar_wait_bounded(bar, phase);
      }
      __threadfence_block();
      named_sync(BAR_CHAIN, THREADS);
    }
    // ---- flush: accumulator row m holds delta term 0 (m < 48) or 1 (48 <= m < 96) of
    // output o = m % 48; per input block, columns c and 32 + c hold activation terms 0
    // and 1 of input c.  Rows of both delta terms add into the same gradient entries.
    if (chain && ok && !first) {
      const int o = r < FD ? r : r - FD;
      const bool row = r < 2 * FD;
#pragma unroll
      for (int l = 0; l < NL; ++l) {
#pragma unroll
        for (int b = 0; b < NBLK(l); ++b) {
          float u[16];
          tc::ld_32x32b_x16(tmem + lane + DWCOL(l) + 64 * b + 16 * h, v);
          tc::ld_32x32b_x16(tmem + lane + DWCOL(l) + 64 * b + 32 + 16 * h, u);
          tc::ld_wait();
          if (row && o < OUT(l)) {
#pragma unroll
            for (int i = 0; i < 16; ++i) {
              const int c = 32 * b + 16 * h + i;
              if (c < IN(l)) atomicAdd(a.grad_params + a.w_off[l] + c * OUT4(l) + o, v[i] + u[i]);
            }
            // layer 3's bias gradient: the PE block's column of ones
            if (l == 3 && b == 1 && h == 1)
              atomicAdd(a.grad_params + a.b_off[l] + o, v[PE_ONES - 16] + u[PE_ONES - 16]);
          }
        }
        if (l != 3 && h == 0) {
          tc::ld_32x32b_x16(tmem + lane + DBCOL(l), v);
          tc::ld_wait();
          if (row && o < OUT(l)) atomicAdd(a.grad_params + a.b_off[l] + o, v[0]);
        }
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tmem, TMEM_COLS);
}

}  // namespace bws
}  // namespace dv

using namespace dv;

extern "C" {

int dv_decode_bwd_tc_split(int kind, int channels, const void* wb, int wb_term_bytes, const int* b_layers,
                           int n_layers, int nvx, int nvy, int nvz, const float* seg, const int* seg_ray,
                           long long n_seg, const int64_t* n_seg_dev, const float* pe_feat, const float* d4,
                           const void* saved, long long saved_bytes, const float* out4, float* grad_voxels,
                           float* grad_params, unsigned char* touched, int* err, void* stream) {
  using namespace dv::bws;
  DV_CHECK(n_seg >= 0, DV_ERR_ARG);
  DV_CHECK(kind == 32 && channels == 32 && n_layers == NL, DV_ERR_UNSUPPORTED);
  if (n_seg == 0) return DV_OK;
  DV_CHECK(wb && b_layers && seg && seg_ray && pe_feat && d4 && saved && out4 && grad_voxels && grad_params,
           DV_ERR_ARG);
  DV_CHECK(nvx > 0 && nvy > 0 && nvz > 0 && wb_term_bytes > 0 && wb_term_bytes % 16 == 0, DV_ERR_ARG);
  DV_CHECK(((uintptr_t)wb & 15) == 0 && ((uintptr_t)saved & 15) == 0 && ((uintptr_t)out4 & 15) == 0 &&
               ((uintptr_t)grad_voxels & 15) == 0 && ((uintptr_t)d4 & 15) == 0,
           DV_ERR_ARG);
  DV_CHECK((n_seg + 127) / 128 * (long long)RECORD <= saved_bytes, DV_ERR_ARG);
  Args a{};
  a.nvx = nvx;
  a.nvy = nvy;
  a.nvz = nvz;
  a.seg = seg;
  a.seg_ray = seg_ray;
  a.S = n_seg;
  a.S_dev = n_seg_dev;
  a.pe_feat = pe_feat;
  a.d4 = reinterpret_cast<const float4*>(d4);
  a.out4 = reinterpret_cast<const float4*>(out4);
  a.saved = reinterpret_cast<const uint8_t*>(saved);
  a.grad_grid = grad_voxels;
  a.grad_params = grad_params;
  a.touched = touched;
  a.wb = reinterpret_cast<const uint8_t*>(wb);
  a.wterm = wb_term_bytes;
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
  // transposed images [N = in][K = out padded to 16], inside one term
  const int bK[NL] = {W, W, W + 16, W, 16}, bN[NL] = {C, W, W, W, W};
  for (int l = 0; l < NL; ++l) {
    a.b_img[l] = b_layers[3 * l];
    DV_CHECK(b_layers[3 * l + 1] == bK[l] && b_layers[3 * l + 2] == bN[l] && bK[l] == KPROP(l), DV_ERR_ARG);
    DV_CHECK(a.b_img[l] % 16 == 0 && a.b_img[l] >= 0, DV_ERR_ARG);
    DV_CHECK((long long)a.b_img[l] + (long long)bK[l] * bN[l] * 2 <= wb_term_bytes, DV_ERR_ARG);
  }
  const Layout lay = Layout::make();
  const size_t smem = lay.bytes();
  auto k = decode_bwd_tc_split_kernel;
  int dev = 0, sms = 0, smem_max = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  DV_CHECK((long long)smem <= (long long)smem_max, DV_ERR_UNSUPPORTED);
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return DV_ERR_CUDA;
  const long long tiles = (n_seg + 127) / 128;
  const long long grid = std::min<long long>(tiles, (long long)sms);
  k<<<(unsigned)grid, THREADS, smem, (cudaStream_t)stream>>>(a);
  DV_TRY_LAUNCH();
  return DV_OK;
}

}  // extern "C"
