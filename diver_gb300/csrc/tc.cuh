// Blackwell (sm_103a) tensor-core primitives as inline PTX: TMEM allocation,
// tcgen05.mma (kind::f16, A and B from shared memory, FP32 accumulators in
// TMEM), tcgen05.commit to an mbarrier, tcgen05.ld of accumulator rows, and
// bounded mbarrier waits.
//
// Operand layout: K-major, no swizzle.  An [R][K] tile (R rows, K a multiple
// of 8 elements of 2 bytes) is stored as 8x8 core matrices of 128 contiguous
// bytes (8 rows x 16 bytes); core matrix (r/8, k/8) sits at
//   (r/8) * SBO + (k/8) * LBO,  LBO = 128 bytes, SBO = (K/8) * 128 bytes,
// and element (r, k) at that base + (r%8)*16 + (k%8)*2.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace dv {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Byte offset of element (r, k) in a K-major no-swizzle tile with K columns.
__host__ __device__ __forceinline__ uint32_t kmajor_offset(int r, int k, int K) {
  return (uint32_t)(((r >> 3) * (K >> 3) + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// Shared-memory matrix descriptor (tcgen05 form: bits 46-48 = 0b001).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFF) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= 1ull << 46;
  return d;  // base offset 0, LBO mode 0, no swizzle
}

// The descriptor of an operand `bytes` further on (a multiple of 16): the
// start address is the low field (address / 16, 14 bits), and shared-memory
// addresses stay below 256 KiB, so the add never carries out of it.
__device__ __forceinline__ uint64_t desc_plus(uint64_t d, uint32_t bytes) { return d + (bytes >> 4); }

// Instruction descriptor for kind::f16: D FP32, A/B both BF16 (bf16 = 1) or
// both FP16 (bf16 = 0), both K-major, shape M x N.
__host__ __device__ __forceinline__ uint32_t idesc_f16(int M, int N, int bf16) {
  return (1u << 4) | ((uint32_t)bf16 << 7) | ((uint32_t)bf16 << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for the given phase parity with an iteration limit; returns false if
// the limit ran out (the caller records an error and stops issuing work).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t limit = 1u << 26) {
  for (uint32_t i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// ---- bulk (non-tensor) async copies between global and shared memory ----
// Both addresses 16-byte aligned, size a multiple of 16 bytes.

// Shared -> global, tracked by this thread's bulk async-group.
__device__ __forceinline__ void bulk_store(void* gdst, const void* ssrc, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst), "r"(smem_u32(ssrc)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// Waits until every committed bulk store of this thread has finished reading shared memory.
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// Waits until every committed bulk store of this thread has completed.
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// Global -> shared, completing `bytes` of transaction count on the mbarrier.
__device__ __forceinline__ void bulk_load(void* sdst, const void* gsrc, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(sdst)),
               "l"(gsrc), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
// One arrival on the mbarrier that also expects `bytes` of transactions.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// Makes generic-proxy shared-memory writes visible to the tensor core.
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// TMEM allocation by one full warp; the base address is written to *dst.
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T, one instruction (K = 16 for kind::f16).
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                        uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Arrives on the mbarrier once all previously issued MMAs of this thread complete.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// 32 lanes x 32 columns: this thread gets row (lane base + laneid), 32 values.
__device__ __forceinline__ void ld_32x32b_x32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void ld_32x32b_x16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void ld_32x32b_x4(uint32_t taddr, float* v) {
  uint32_t r[4];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(taddr)
               : "memory");
#pragma unroll
  for (int i = 0; i < 4; ++i) v[i] = __uint_as_float(r[i]);
}

// Packs two floats into a bf16x2 / f16x2 word (low half = a).
template <int BF16>
__device__ __forceinline__ uint32_t pack2(float a, float b) {
  uint32_t r;
  if (BF16)
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(b), "f"(a));
  else
    asm("cvt.rn.f16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(b), "f"(a));
  return r;
}

// Low / high BF16 element of a bf16x2 word as a float.
__device__ __forceinline__ float bf_lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf_hi(uint32_t w) { return __uint_as_float(w & 0xffff0000u); }

// FP32 pair (a, b) as a sum of TERMS BF16 pairs: w[0] = RN(a, b), then each
// further term rounds what the previous ones left.  Every residual is exact in
// FP32 (a minus its value rounded to 8 significant bits keeps only a's low
// bits), so the terms sum to (a, b) within 2^-8 (one term), 2^-16 (two) or
// 2^-24 (three) of its magnitude.  A product of two such sums, taken as the
// BF16 products whose term indices add up to at most TERMS - 1 (1, 3 or 6
// tensor-core MMAs), keeps that precision: the split-operand ("BF16x3",
// "BF16x6") emulation of FP32 products on BF16 tensor cores.
template <int TERMS>
__device__ __forceinline__ void split_pair(float a, float b, uint32_t* w) {
  w[0] = pack2<1>(a, b);
#pragma unroll
  for (int i = 1; i < TERMS; ++i) {
    a = __fsub_rn(a, bf_lo(w[i - 1]));
    b = __fsub_rn(b, bf_hi(w[i - 1]));
    w[i] = pack2<1>(a, b);
  }
}

// Residency of a persistent kernel whose CTAs each allocate `ncols` TMEM
// columns.  Registers and shared memory may admit more CTAs per SM than the
// 512 TMEM columns can hold; a CTA scheduled beyond that waits inside
// tcgen05.alloc until a resident CTA has finished its whole share of the
// tiles, which stretches that SM to about twice the others.  The dynamic
// shared memory is therefore padded until shared memory alone admits no more
// CTAs than the TMEM does, and the kernel asks for the largest shared-memory
// carveout so that the padded count is what the SM really holds.
struct Residency {
  int per_sm;       // CTAs per SM the launch may count on (>= 1)
  size_t dyn_smem;  // dynamic shared memory to launch with (>= the request)
};

inline Residency tmem_residency(const void* kernel, size_t dyn_smem, int ncols, int threads) {
  Residency r{1, dyn_smem};
  cudaFuncAttributes fa{};
  if (cudaFuncGetAttributes(&fa, kernel) != cudaSuccess) return r;
  int dev = 0, regs_sm = 65536, smem_sm = 228 * 1024, thr_sm = 2048, reserved = 1024;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
  cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  cudaDeviceGetAttribute(&thr_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev);
  cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
  const size_t fixed = fa.sharedSizeBytes + (size_t)reserved;
  const int by_threads = thr_sm / threads;
  const int by_regs = regs_sm / (fa.numRegs > 0 ? fa.numRegs * threads : threads);
  const int by_smem = (int)(smem_sm / (dyn_smem + fixed));
  const int by_tmem = 512 / ncols;
  int n = by_threads < by_regs ? by_threads : by_regs;
  n = n < by_tmem ? n : by_tmem;
  if (n >= by_smem) {
    r.per_sm = by_smem > 0 ? by_smem : 1;
    return r;
  }
  // Pad: (n + 1) CTAs must no longer fit, n still must.
  size_t per_cta = (size_t)smem_sm / (size_t)(n + 1) + 1;
  size_t dyn = per_cta > fixed ? per_cta - fixed : 0;
  dyn = (dyn + 127) / 128 * 128;
  if (dyn < dyn_smem) dyn = dyn_smem;
  if ((size_t)n * (dyn + fixed) > (size_t)smem_sm) {
    r.per_sm = by_smem < by_tmem ? by_smem : by_tmem;  // cannot pad exactly; stay within both limits
    return r;
  }
  r.per_sm = n;
  r.dyn_smem = dyn;
  return r;
}

}  // namespace tc
}  // namespace dv
