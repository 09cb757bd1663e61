// Tensor-core (tcgen05) backward of the DIVeR32 decoder with split BF16
// operands: FP32-grade gradients from BF16 tensor cores.
//
// Every FP32 operand is carried as a sum of BF16 terms (tc::split_pair):
//   - delta propagation  dL/d input = delta @ W: delta and W as three terms
//     each, the six products whose term indices add up to at most 2;
//   - weight gradient    dW += delta^T @ activation: two terms each, three
//     products (FP32 accumulators resident in TMEM for the CTA's life);
//   - bias gradient      dB += delta^T @ ones: the column sums of the two-term
//     delta as two more products per layer, also accumulated in TMEM.
// Products are accumulated in FP32 in TMEM, so the propagated deltas and the
// gradients keep about 2^-24 (propagation) and 2^-16 (weight gradients) of
// relative precision per product; emulating the kernel's arithmetic on the
// CPU gives gradients within a few 1e-7 (grid) and 1e-6 (weights) relative
// of an FP64 backward, where a single BF16 term gives 1e-2.
//
// The forward is not recomputed: dv_decode_fwd_tc_split saved, per tile of 128
// segments, every layer's input as two BF16 terms (X0, A1, A2, hidden, A4;
// 16 KiB each), and its FP32 out4 gives the colour logits' sigmoid.  The
// record is read into shared memory by bulk async copies, one per layer slot.
//
// One CTA per SM, 384 threads in two groups (see the kernel): 256 chain
// threads, where thread t owns segment row r = t % 128 (TMEM lane r; warps w
// and w + 4 share a lane quadrant) and half h = t / 128 of each row's columns
// in the epilogues, and 128 scatter threads.  Shared memory (about 184 KiB):
// transposed weight images in three terms, the saved record in five per-layer
// slots, the PE tile in two terms, the delta tile in three terms (48 columns:
// the widest propagation K), a tile of ones and the FP32 staging rows of the
// feature gradient.  TMEM: all 512 columns (working, weight and bias gradients).  The weight-gradient MMA reads the delta tile transposed with
// M = 128 output rows; rows past a layer's outputs read the neighbouring
// (finite) data of the tile and of the next term and land in TMEM rows that
// are never read.
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
constexpr int CHAIN = 256;             // threads of the layer chain (warps 0-7)
constexpr int THREADS = CHAIN + 128;   // + one warpgroup for the corner scatter
constexpr int FD = 48;              // delta tile columns (K of the widest propagation MMA)
constexpr int TILE = 128 * 32 * 2;  // one term of a [128][32] BF16 tile
constexpr int DTILE = 128 * FD * 2; // one term of the delta tile
constexpr int TMEM_COLS = 512;     // 64 working + 192 weight-gradient + 80 bias-gradient columns, rounded up
// layer: 0 (C->W), 1 (W->W), 2 (W->W+1: sigma, hidden), 3 (W+27->W), 4 (W->3)
__host__ __device__ constexpr int IN(int l) { return l == 0 ? C : (l == 3 ? W + PE_DIM : W); }
__host__ __device__ constexpr int OUT(int l) { return l == 2 ? W + 1 : (l == 4 ? 3 : W); }
__host__ __device__ constexpr int OUT4(int l) { return pad4(OUT(l)); }
__host__ __device__ constexpr int NIN(int l) { return l == 3 ? 64 : 32; }  // weight-gradient columns (in, padded)
__host__ __device__ constexpr int DWCOL(int l) { return l == 0 ? 64 : (l <= 3 ? DWCOL(l - 1) + NIN(l - 1) : 224); }
__host__ __device__ constexpr int DBCOL(int l) { return 256 + 16 * l; }  // bias gradient of layer l (column 0 of 16)
__host__ __device__ constexpr int KPROP(int l) { return l == 4 ? 16 : (l == 2 ? W + 16 : W); }  // propagation K
constexpr uint32_t RECORD = 5 * 2 * TILE;  // saved record of one tile: 5 layer inputs x 2 terms
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
  int w_off[NL], b_off[NL];
  const uint8_t* wb;     // transposed weight images, three terms of wterm bytes
  int wterm;
  int b_img[NL];         // byte offset of layer l's image inside a term
  int* err;
};

// Shared-memory layout (byte offsets; wterm = 10240 for DIVeR32).
struct Layout {
  uint32_t bb, rec, pe, d, ones, stage, bar;
  __host__ __device__ static Layout make(int wterm) {
    Layout L;
    L.bb = 0;
    L.rec = (uint32_t)(3 * wterm + 1023) / 1024 * 1024;
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

// Writes n values (multiple of 8) of row r, starting at column c0, as three
// BF16 terms of a K-major tile with F columns (term i at tile + i * tstride).
__device__ __forceinline__ void put3(uint8_t* tile, uint32_t tstride, int F, int r, int c0, const float* v, int n) {
#pragma unroll
  for (int c = 0; c < n; c += 8) {
    uint32_t x[3], y[3], z[3], u[3];
    tc::split_pair<3>(v[c], v[c + 1], x);
    tc::split_pair<3>(v[c + 2], v[c + 3], y);
    tc::split_pair<3>(v[c + 4], v[c + 5], z);
    tc::split_pair<3>(v[c + 6], v[c + 7], u);
    uint8_t* dst = tile + tc::kmajor_offset(r, c0 + c, F);
#pragma unroll
    for (int i = 0; i < 3; ++i) *reinterpret_cast<uint4*>(dst + i * tstride) = make_uint4(x[i], y[i], z[i], u[i]);
  }
}

// Same with two terms.
__device__ __forceinline__ void put2(uint8_t* tile, uint32_t tstride, int F, int r, int c0, const float* v, int n) {
#pragma unroll
  for (int c = 0; c < n; c += 8) {
    uint32_t x[2], y[2], z[2], u[2];
    tc::split_pair<2>(v[c], v[c + 1], x);
    tc::split_pair<2>(v[c + 2], v[c + 3], y);
    tc::split_pair<2>(v[c + 4], v[c + 5], z);
    tc::split_pair<2>(v[c + 6], v[c + 7], u);
    uint8_t* dst = tile + tc::kmajor_offset(r, c0 + c, F);
#pragma unroll
    for (int i = 0; i < 2; ++i) *reinterpret_cast<uint4*>(dst + i * tstride) = make_uint4(x[i], y[i], z[i], u[i]);
  }
}

// Zeroes v[i] where the activation (leading term of a [128][32] tile, row r,
// columns c0..c0+n-1) is not positive: the ReLU derivative.  The leading
// BF16 term has the sign of the FP32 activation (and is zero only with it).
__device__ __forceinline__ void relu_mask(const uint8_t* tile, int r, int c0, float* v, int n) {
#pragma unroll
  for (int c = 0; c < n; c += 8) {
    const uint4 w = *reinterpret_cast<const uint4*>(tile + tc::kmajor_offset(r, c0 + c, 32));
    const uint32_t x[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (!(tc::bf_lo(x[j]) > 0.f)) v[c + 2 * j] = 0.f;
      if (!(tc::bf_hi(x[j]) > 0.f)) v[c + 2 * j + 1] = 0.f;
    }
  }
}

// Propagation: TMEM[0..N) = delta [128][K] (three terms, K-major, FD
// columns) x image^T (image [N][K], three terms of wterm bytes).
__device__ __forceinline__ void mma_prop(uint32_t tmem, const uint8_t* D, const uint8_t* img, int wterm, int K, int N) {
  constexpr int PA6[6] = {0, 0, 1, 0, 2, 1};  // term of delta, per product
  constexpr int PB6[6] = {0, 1, 0, 2, 0, 1};  // term of the weights
  const uint32_t idesc = tc::idesc_f16(128, N, 1);
#pragma unroll
  for (int p = 0; p < 6; ++p) {
    const uint32_t a0 = tc::smem_u32(D + PA6[p] * DTILE), b0 = tc::smem_u32(img + PB6[p] * wterm);
    for (int k = 0; k < K / 16; ++k)
      tc::mma_f16(tmem, tc::smem_desc(a0 + k * 256, 128, (FD / 8) * 128),
                  tc::smem_desc(b0 + k * 256, 128, (uint32_t)(K / 8) * 128), idesc, (p > 0 || k > 0) ? 1u : 0u);
  }
}

// Weight gradient over the tile's 128 segments: TMEM dW[128 = out][32 = in]
// += delta^T x act, both MN-major views of row tiles (two terms each; the
// activation tile [128][32], term stride TILE).
__device__ __forceinline__ void mma_dw(uint32_t tmem, const uint8_t* D, const uint8_t* act, bool accumulate) {
  const uint32_t idesc = tc::idesc_f16(128, 32, 1) | (1u << 15) | (1u << 16);
  constexpr uint32_t lboA = (FD / 8) * 128, lboB = (32 / 8) * 128;
  constexpr int PA3[3] = {0, 0, 1};  // term of delta, per product
  constexpr int PB3[3] = {0, 1, 0};  // term of the activation
#pragma unroll
  for (int p = 0; p < 3; ++p) {
    const uint32_t a0 = tc::smem_u32(D + PA3[p] * DTILE), b0 = tc::smem_u32(act + PB3[p] * TILE);
    for (int k = 0; k < 8; ++k)
      tc::mma_f16(tmem, tc::smem_desc(a0 + k * 2 * lboA, lboA, 128), tc::smem_desc(b0 + k * 2 * lboB, lboB, 128),
                  idesc, (accumulate || p > 0 || k > 0) ? 1u : 0u);
  }
}

// Bias gradient over the tile's 128 segments: TMEM dB[128 = out][16] += delta^T x
// ones, i.e. every column of dB is the column sum of the delta (two terms, two
// products; the ones are exact in BF16).  The ones tile is all ones, so any
// reading of its layout is the same.
__device__ __forceinline__ void mma_db(uint32_t tmem, const uint8_t* D, const uint8_t* ones, bool accumulate) {
  const uint32_t idesc = tc::idesc_f16(128, 16, 1) | (1u << 15) | (1u << 16);
  constexpr uint32_t lboA = (FD / 8) * 128, lboB = (16 / 8) * 128;
  const uint32_t b0 = tc::smem_u32(ones);
#pragma unroll
  for (int p = 0; p < 2; ++p) {
    const uint32_t a0 = tc::smem_u32(D + p * DTILE);
    for (int k = 0; k < 8; ++k)
      tc::mma_f16(tmem, tc::smem_desc(a0 + k * 2 * lboA, lboA, 128), tc::smem_desc(b0 + k * 2 * lboB, lboB, 128),
                  idesc, (accumulate || p > 0 || k > 0) ? 1u : 0u);
  }
}

// Named barriers of the two thread groups (barrier 0 is __syncthreads).
constexpr int BAR_CHAIN = 1;       // the 256 chain threads among themselves
constexpr int BAR_STAGE_FULL = 2;  // chain -> scatter: a tile's feature gradients are staged
constexpr int BAR_STAGE_FREE = 3;  // scatter -> chain: the staging rows may be overwritten

__device__ __forceinline__ void named_sync(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }
__device__ __forceinline__ void named_arrive(int id, int n) {
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(n) : "memory");
}
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
  named_sync(BAR_CHAIN, CHAIN);
}

// PE tile row r, columns 16h..16h+15 (PE_DIM = 27 values, zeros after), two terms.
__device__ __forceinline__ void write_pe(const Args& a, uint8_t* PE, int ray, int r, int h) {
  float v[16];
  const float* pf = a.pe_feat + (long long)ray * PE_PAD + 16 * h;
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = (16 * h + i < PE_DIM) ? __ldg(pf + i) : 0.f;
  put2(PE, TILE, 32, r, 16 * h, v, 16);
}

// Delta of the colour logits (dL/drgb * sigmoid') into columns 0..15 of row r.
__device__ __forceinline__ void write_delta4(uint8_t* D, int r, float4 g, float4 oc) {
  float v[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = 0.f;
  v[0] = g.y * oc.y * (1.f - oc.y);
  v[1] = g.z * oc.z * (1.f - oc.z);
  v[2] = g.w * oc.w * (1.f - oc.w);
  put3(D, DTILE, FD, r, 0, v, 16);
}

// One tile per step of the persistent loop, in two concurrent groups:
//   chain   (warps 0-7)  the five layer steps: per layer, the propagation and
//                        weight-gradient MMAs, the bias column sums and the
//                        epilogue that forms the next delta; it stages the
//                        tile's feature gradient (FP32) for the scatter group
//   scatter (warps 8-11) the previous tile's feature gradient into the 8
//                        corner rows of every segment (vector atomics)
// The saved record sits in five per-layer slots, each with its own mbarrier:
// when a layer step of tile i is done with its slot, that slot is refilled
// with tile i + gridDim.x's layer input, so the next tile's loads run behind
// the rest of this tile.  The PE tile and the first delta of the next tile are
// also written as soon as this tile is done with them.
__global__ void __launch_bounds__(THREADS, 1) decode_bwd_tc_split_kernel(const Args a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  const Layout lay = Layout::make(a.wterm);
  uint8_t* Bb = smem + lay.bb;
  uint8_t* REC = smem + lay.rec;
  uint8_t* PE = smem + lay.pe;
  uint8_t* D = smem + lay.d;
  uint8_t* ONES = smem + lay.ones;
  float* stage = reinterpret_cast<float*>(smem + lay.stage);  // [128][C + 4] FP32
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + lay.bar);
  uint64_t* bar_rec = bar + 1;  // [NL]: completion of slot l's record load
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 1 + NL);
  int* abort_flag = reinterpret_cast<int*>(tslot + 1);

  const int t = threadIdx.x, warp = t >> 5;
  const bool chain = t < CHAIN;
  const int r = t & 127, h = (t >> 7) & 1;
  const long long S = segment_total(a.S, a.S_dev);
  const long long tiles = (S + 127) / 128;

  for (int i = t; i < 3 * a.wterm / 16; i += THREADS)
    reinterpret_cast<uint4*>(Bb)[i] = __ldg(reinterpret_cast<const uint4*>(a.wb) + i);
  for (int i = t; i < 3 * DTILE / 16; i += THREADS) reinterpret_cast<uint4*>(D)[i] = make_uint4(0, 0, 0, 0);
  for (int i = t; i < (int)ONES_BYTES / 16; i += THREADS)
    reinterpret_cast<uint4*>(ONES)[i] = make_uint4(0x3f803f80u, 0x3f803f80u, 0x3f803f80u, 0x3f803f80u);  // bf16 1.0
  if (t == 0) {
    tc::mbar_init(bar, 1);
    for (int l = 0; l < NL; ++l) tc::mbar_init(bar_rec + l, 1);
    *abort_flag = 0;
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

  if (!chain) {
    // ---------------- scatter group ----------------
    const int u = t - CHAIN;  // 0..127
    constexpr int TPS = C / 4;
    if (blockIdx.x < tiles) named_arrive(BAR_STAGE_FREE, THREADS);  // the staging rows start free
    for (long long tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
      named_sync(BAR_STAGE_FULL, THREADS);
      if (*reinterpret_cast<volatile int*>(abort_flag)) break;
#pragma unroll 1
      for (int i = u; i < 128 * TPS; i += 128) {
        const int ls = i / TPS, q = i % TPS;
        const long long ss = tile * 128 + ls;
        if (ss < S) {
          const float* sg = a.seg + ss * 6;
          const SegCorner sc = segment_corners(__ldg(sg), __ldg(sg + 1), __ldg(sg + 2), __ldg(sg + 3),
                                               __ldg(sg + 4), __ldg(sg + 5), a.nvx, a.nvy, a.nvz);
          const float4 gf = *reinterpret_cast<const float4*>(stage + ls * (C + 4) + 4 * q);
          scatter4(a.grad_grid, sc, C, q, gf, a.nvx, a.nvy);
        }
      }
      __threadfence_block();
      if (tile + gridDim.x < tiles) named_arrive(BAR_STAGE_FREE, THREADS);
    }
  } else {
    // ---------------- chain group ----------------
    const uint32_t lane = (uint32_t)((warp & 3) * 32) << 16;
    const uint32_t trow = tmem + lane;
    uint32_t phase = 0, phase_rec = 0;  // phase_rec: bit l = parity of slot l's next completion
    uint32_t pending = 0;               // thread 0: slots with a load in flight
    bool mma_inflight = false;          // thread 0: an MMA batch committed and not yet waited for
    bool ok = true, first = true;
    float v[32];
    // the CTA's first tile: record loads, PE tile, first delta
    long long tile = blockIdx.x;
    if (tile < tiles) {
      if (t == 0) {
        const uint8_t* rec = a.saved + tile * (long long)RECORD;
        for (int l = 0; l < NL; ++l) {
          tc::mbar_arrive_expect_tx(bar_rec + l, 2 * TILE);
          tc::bulk_load(REC + l * 2 * TILE, rec + l * 2 * TILE, 2 * TILE, bar_rec + l);
        }
        pending = (1u << NL) - 1;
      }
      const long long s = tile * 128 + r;
      const bool valid = s < S;
      write_pe(a, PE, valid ? __ldg(a.seg_ray + s) : 0, r, h);
      if (h == 0)
        write_delta4(D, r, valid ? a.d4[s] : make_float4(0.f, 0.f, 0.f, 0.f),
                     valid ? a.out4[s] : make_float4(0.f, 0.f, 0.f, 0.f));
    }
    for (; tile < tiles && ok; tile += gridDim.x) {
      const long long s = tile * 128 + r;
      const bool valid = s < S;
      const long long next = tile + gridDim.x;
      const long long sn = next * 128 + r;
      const bool valid_next = next < tiles && sn < S;
      const float gx = valid ? a.d4[s].x : 0.f;  // dL/dsigma of this row (layer 2's delta)
      chain_sync();  // the PE tile and the first delta are in place
      // layers last to first (unrolled: every layer constant is a compile-time value)
#pragma unroll
      for (int l = NL - 1; l >= 0; --l) {
        const uint8_t* act = REC + l * 2 * TILE;  // this layer's input, two terms TILE apart
        // this layer's record slot has arrived (bounded wait; the parities
        // advance only on success: after a timeout the abort path waits with them)
        const bool arrived = tc::mbar_wait_bounded(bar_rec + l, (phase_rec >> l) & 1u);
        if (arrived) phase_rec ^= 1u << l;
        if (t == 0 && arrived) {
          pending &= ~(1u << l);
          tc::fence_after_sync();
          mma_prop(tmem, D, Bb + a.b_img[l], a.wterm, KPROP(l), l == 0 ? C : W);
          if (l == 3) {
            mma_dw(tmem + DWCOL(3), D, act, !first);
            mma_dw(tmem + DWCOL(3) + 32, D, PE, !first);
          } else {
            mma_dw(tmem + DWCOL(l), D, act, !first);
          }
          mma_db(tmem + DBCOL(l), D, ONES, !first);
          tc::mma_commit(bar);
          mma_inflight = true;
        }
        // if thread 0's slot wait gave up it issued nothing: every thread's MMA wait then
        // runs out too, and the AND below stops them all
        bool done = false;
        if (arrived) {
          done = tc::mbar_wait_bounded(bar, phase);
          if (done) {
            phase ^= 1u;
            if (t == 0) mma_inflight = false;
          }
        }
        tc::fence_after_sync();
        ok = named_and(BAR_CHAIN, CHAIN, arrived && done);
        if (!ok) break;
        if (l == 3) {
          // delta of layer 2: (dL/dsigma, d hidden[0..31]) in columns 0..32, zeros to 47;
          // half 0 writes columns 0..23, half 1 columns 24..47
          tc::ld_32x32b_x32(trow, v);
          tc::ld_wait();
          float w[24];
          if (h == 0) {
            w[0] = gx;
#pragma unroll
            for (int i = 1; i < 24; ++i) w[i] = v[i - 1];
          } else {
#pragma unroll
            for (int i = 0; i < 24; ++i) w[i] = (i + 23 < W) ? v[i + 23] : 0.f;
          }
          put3(D, DTILE, FD, r, 24 * h, w, 24);
          // this tile's PE is consumed: the next tile's goes in now
          if (next < tiles) write_pe(a, PE, valid_next ? __ldg(a.seg_ray + sn) : 0, r, h);
        } else if (l > 0) {
          tc::ld_32x32b_x16(trow + 16 * h, v);
          tc::ld_wait();
          relu_mask(act, r, 16 * h, v, 16);  // this layer's input is relu of the previous layer's output
          put3(D, DTILE, FD, r, 16 * h, v, 16);
        } else {
          // dL/dfeature (FP32) to the staging rows once the scatter group is done with them
          float4 gn = make_float4(0.f, 0.f, 0.f, 0.f), on = gn;
          if (valid_next && h == 0) {
            gn = a.d4[sn];
            on = a.out4[sn];
          }
          tc::ld_32x32b_x16(trow + 16 * h, v);
          tc::ld_wait();
          named_sync(BAR_STAGE_FREE, THREADS);
          float* st = stage + r * (C + 4) + 16 * h;
#pragma unroll
          for (int i = 0; i < 16; i += 4)
            *reinterpret_cast<float4*>(st + i) =
                valid ? make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]) : make_float4(0.f, 0.f, 0.f, 0.f);
          __threadfence_block();
          named_arrive(BAR_STAGE_FULL, THREADS);
          // this tile's deltas are consumed: the next tile's first delta goes in now
          if (next < tiles && h == 0) write_delta4(D, r, gn, on);
        }
        chain_sync();  // D is complete for the next layer; every read of this layer's slot is done
        if (t == 0 && next < tiles) {
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
    if (!ok) {
      if (t == 0) {
        if (a.err) atomicExch(a.err, 1);
        *reinterpret_cast<volatile int*>(abort_flag) = 1;
        // record loads and MMAs still in flight complete before the CTA frees
        // its shared memory and TMEM (bounded waits)
        for (int l = 0; l < NL; ++l)
          if ((pending >> l) & 1u) tc::mbar_wait_bounded(bar_rec + l, (phase_rec >> l) & 1u);
        if (mma_inflight) tc::mbar_wait_bounded(bar, phase);
      }
      __threadfence_block();
      named_sync(BAR_CHAIN, CHAIN);
      named_arrive(BAR_STAGE_FULL, THREADS);  // wakes the scatter group, which sees the flag and stops
    }
    // ---- flush: weight gradients from TMEM (row o = out index = this thread's lane) ----
    if (ok && !first) {
#pragma unroll
      for (int l = 0; l < NL; ++l) {
        const int o = r;
#pragma unroll
        for (int c0 = 0; c0 < NIN(l); c0 += 32) {
          tc::ld_32x32b_x16(tmem + lane + DWCOL(l) + c0 + 16 * h, v);
          tc::ld_wait();
          if (o < OUT(l)) {
#pragma unroll
            for (int i = 0; i < 16; ++i) {
              const int c = c0 + 16 * h + i;
              if (c < IN(l)) atomicAdd(a.grad_params + a.w_off[l] + c * OUT4(l) + o, v[i]);
            }
          }
        }
        if (h == 0) {
          tc::ld_32x32b_x16(tmem + lane + DBCOL(l), v);
          tc::ld_wait();
          if (o < OUT(l)) atomicAdd(a.grad_params + a.b_off[l] + o, v[0]);
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
                           float* grad_params, int* err, void* stream) {
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
  const Layout lay = Layout::make(wb_term_bytes);
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
