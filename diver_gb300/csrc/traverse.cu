// Voxel traversal kernels: dense and masked 3D-DDA (training/offline path),
// the octree first-hit search and the 8-hit ray march (real-time path), and
// the prefix sum that turns per-ray counts into CSR segment offsets.
//
// One thread walks one ray; the walk itself is inherently sequential (each
// crossing is computed from the previous, rounded point), so bit-exactness
// with the reference fixes the per-ray order of operations.  What changes
// against the reference is around the walk: outputs are either counted only,
// written to caller-sized padded rows, or written compacted (CSR) so that the
// segment-parallel decoder never touches padding; max(count) is reduced per
// warp before one atomic; launches are stream-ordered with no device sync.
#include "common.cuh"
#include "scan.cuh"

namespace dv {

// WALK_SLOTS: one walk both counts and writes, each ray into its own fixed
// range of `slot` rows (b * slot ...), compacted into CSR lists afterwards.
enum WalkMode { WALK_COUNT = 0, WALK_PADDED = 1, WALK_SEGMENTS = 2, WALK_SLOTS = 3 };

struct WalkArgs {
  int batch;
  int max_n;
  float xyzmin;
  float n;
  float3 o3;        // per-axis grid origin (world)
  float3 n3;        // per-axis extent in voxels
  int mx, my;       // occupancy cells along x and y (masked walk)
  float voxel_size;
  float mask_scale;
  int m;            // occupancy cells per side
  long long cells;  // m^3
  bool fast;        // grid small enough for the reciprocal-based division (< 2^22 voxels per side)
  const float* o;
  const float* v;
  const uint8_t* mask;
  float* inter;
  int* num;
  float* tns;
  int* max_count;
  int* last_step;          // count: per ray, the walk step (1-based) of its last occupied voxel, 0 if none
  const int* stop_step;    // segments: per ray, the step after which the walk may stop (last_step of the count)
  long long slot;          // slots: rows per ray
  const int64_t* offsets;
  float* seg;
  float* seg_t;
  int* seg_ray;
};

__device__ __forceinline__ void warp_max_atomic(int* dst, int value, bool active) {
  const unsigned full = __activemask();
  const int mx = __reduce_max_sync(full, active ? value : 0);
  if (dst != nullptr && (threadIdx.x & 31) == (__ffs(full) - 1)) atomicMax(dst, mx);
}

__device__ __forceinline__ float3 ray_origin_voxel(const float* o, int b, float xyzmin, float vs) {
  return make_float3(__fdiv_rn(__fsub_rn(__ldg(o + 3 * b + 0), xyzmin), vs),
                     __fdiv_rn(__fsub_rn(__ldg(o + 3 * b + 1), xyzmin), vs),
                     __fdiv_rn(__fsub_rn(__ldg(o + 3 * b + 2), xyzmin), vs));
}

__device__ __forceinline__ float3 ray_origin_voxel3(const float* o, int b, float3 o3, float vs) {
  return make_float3(__fdiv_rn(__fsub_rn(__ldg(o + 3 * b + 0), o3.x), vs),
                     __fdiv_rn(__fsub_rn(__ldg(o + 3 * b + 1), o3.y), vs),
                     __fdiv_rn(__fsub_rn(__ldg(o + 3 * b + 2), o3.z), vs));
}

__device__ __forceinline__ float3 load3(const float* p, int b) {
  return make_float3(__ldg(p + 3 * b + 0), __ldg(p + 3 * b + 1), __ldg(p + 3 * b + 2));
}

__device__ __forceinline__ float3 signs(float3 d) {
  return make_float3(step_sign(d.x), step_sign(d.y), step_sign(d.z));
}

// Dense walk: entry point, then every plane crossing while the point stays
// in [0,n]^3.  Reference ray_voxel_intersect.cu:39-150.
template <int MODE, bool FAST>
__device__ __forceinline__ int dense_walk(const WalkArgs& a, int b, float3 p, const float3 d, float t, float* row,
                                          float* trow, int64_t base, int64_t cap) {
  const float3 s = signs(d);
  const float3 r = FAST ? recip3(d) : d;
  int count = 1;
  float3 q;
  float dt;
  const int step_cap = walk_cap(a.n, a.n, a.n);
  int k = 0;
  for (; k < step_cap; ++k) {
    grid_step<FAST>(p, d, r, s, q, dt);
    const float tq = __fadd_rn(t, dt);
    if (outside_closed(q, a.n)) break;
    if (MODE == WALK_PADDED && count < a.max_n) {
      row[3 * count + 0] = q.x;
      row[3 * count + 1] = q.y;
      row[3 * count + 2] = q.z;
      trow[count] = __fmul_rn(tq, a.voxel_size);
    }
    if (MODE == WALK_SEGMENTS && count - 1 < cap) {
      float2* sg = reinterpret_cast<float2*>(a.seg + (base + count - 1) * 6);
      sg[0] = make_float2(p.x, p.y);
      sg[1] = make_float2(p.z, q.x);
      sg[2] = make_float2(q.y, q.z);
      if (a.seg_t) a.seg_t[base + count - 1] = __fmul_rn(t, a.voxel_size);
      if (a.seg_ray) a.seg_ray[base + count - 1] = b;
    }
    ++count;
    p = q;
    t = tq;
  }
  if (k == step_cap) note_cap_hit();
  return count;
}

template <int MODE>
__global__ void __launch_bounds__(256) dense_walk_kernel(const WalkArgs a) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = b < a.batch;
  int count = 0;
  if (live) {
    const float3 d = load3(a.v, b);
    float3 p = ray_origin_voxel(a.o, b, a.xyzmin, a.voxel_size);
    float t;
    const bool hit = dir_ok(d) && box_entry(p, d, a.n, t);
    float* row = nullptr;
    float* trow = nullptr;
    int64_t base = 0, cap = 0;
    if (MODE == WALK_PADDED) {
      row = a.inter + (long long)b * a.max_n * 3;
      trow = a.tns + (long long)b * a.max_n;
      if (a.max_n > 0) {
        row[0] = p.x;
        row[1] = p.y;
        row[2] = p.z;
      }
    }
    if (MODE == WALK_SEGMENTS) {
      base = a.offsets[b];
      cap = a.offsets[b + 1] - base;
    }
    if (hit) {
      if (MODE == WALK_PADDED && a.max_n > 0) trow[0] = __fmul_rn(t, a.voxel_size);
      count = (a.fast && recip_ok(d)) ? dense_walk<MODE, true>(a, b, p, d, t, row, trow, base, cap)
                          : dense_walk<MODE, false>(a, b, p, d, t, row, trow, base, cap);
    }
    if (MODE != WALK_SEGMENTS) a.num[b] = count;
  }
  if (MODE != WALK_SEGMENTS) warp_max_atomic(a.max_count, count, live);
}

// Segment record writer for the compacted (CSR) output.  A segment at an even
// global index is held back in registers; its successor then goes out with it
// as one 48-byte pair (three aligned 16-byte stores of the six coordinates,
// 8-byte stores of the two t and ray values).  A segment that has no
// successor slot, or that sits at an odd index with nothing held, is written
// alone (8-byte stores).  Needs seg 16-byte and seg_t / seg_ray 8-byte aligned
// buffers, which the entry points check.
struct SegWriter {
  float h[7];  // held segment: entry xyz, exit xyz, t
  int64_t hi;  // its global index, -1 when nothing is held
  __device__ __forceinline__ SegWriter() : hi(-1) {}

  __device__ __forceinline__ void single(const WalkArgs& a, int b, int64_t g, const float* v, float t) {
    float2* sg = reinterpret_cast<float2*>(a.seg + g * 6);
    sg[0] = make_float2(v[0], v[1]);
    sg[1] = make_float2(v[2], v[3]);
    sg[2] = make_float2(v[4], v[5]);
    if (a.seg_t) a.seg_t[g] = t;
    if (a.seg_ray) a.seg_ray[g] = b;
  }

  __device__ __forceinline__ void put(const WalkArgs& a, int b, int64_t g, bool has_next, const float3 p,
                                      const float3 q, float t) {
    if (hi >= 0) {  // g == hi + 1, hi even
      float4* s4 = reinterpret_cast<float4*>(a.seg + hi * 6);
      s4[0] = make_float4(h[0], h[1], h[2], h[3]);
      s4[1] = make_float4(h[4], h[5], p.x, p.y);
      s4[2] = make_float4(p.z, q.x, q.y, q.z);
      if (a.seg_t) *reinterpret_cast<float2*>(a.seg_t + hi) = make_float2(h[6], t);
      if (a.seg_ray) *reinterpret_cast<int2*>(a.seg_ray + hi) = make_int2(b, b);
      hi = -1;
    } else if (((g & 1) == 0) && has_next) {
      h[0] = p.x;
      h[1] = p.y;
      h[2] = p.z;
      h[3] = q.x;
      h[4] = q.y;
      h[5] = q.z;
      h[6] = t;
      hi = g;
    } else {
      const float v[6] = {p.x, p.y, p.z, q.x, q.y, q.z};
      single(a, b, g, v, t);
    }
  }

  __device__ __forceinline__ void flush(const WalkArgs& a, int b) {
    if (hi >= 0) single(a, b, hi, h, h[6]);
    hi = -1;
  }
};

// Masked walk: (entry, exit) of every voxel whose occupancy byte is set.
// Reference ray_voxel_intersect.cu:203-318.
//
// The crossing points form a dependent chain, but the occupancy byte of a
// voxel only decides whether its segment is recorded.  The walk therefore
// runs LOOKAHEAD steps ahead: it computes up to LOOKAHEAD crossings and issues
// their occupancy loads back to back, then records the occupied ones in
// order, so a ray waits for one load latency per LOOKAHEAD voxels instead of
// one per voxel (which bounds small batches, where few warps are resident).
template <int MODE, bool FAST, int LOOKAHEAD>
__device__ __forceinline__ int masked_walk(const WalkArgs& a, int b, float3 p, const float3 d, float t) {
  const float3 s = signs(d);
  const float3 r = FAST ? recip3(d) : d;
  float* row = nullptr;
  float* trow = nullptr;
  int64_t base = 0, cap = 0;
  if (MODE == WALK_PADDED) {
    row = a.inter + (long long)b * a.max_n * 6;
    trow = a.tns + (long long)b * a.max_n;
  }
  if (MODE == WALK_SEGMENTS) {
    base = a.offsets[b];
    cap = a.offsets[b + 1] - base;
  }
  if (MODE == WALK_SLOTS) {
    base = (int64_t)b * a.slot;
    cap = a.slot;
  }
  SegWriter w;
  int count = 0;
  bool done = false;
  // steps taken so far, the step of the last occupied voxel (counting), and
  // where the walk may stop (emitting: nothing occupied lies beyond it)
  int steps = 0, last = 0;
  const int step_cap = walk_cap(a.n3.x, a.n3.y, a.n3.z);
  const int limit = min((MODE == WALK_SEGMENTS && a.stop_step) ? a.stop_step[b] : 0x7fffffff, step_cap);
  bool left = false;  // the walk left the grid
  while (!done) {
    float3 P[LOOKAHEAD + 1];
    float T[LOOKAHEAD];
    uint8_t occ[LOOKAHEAD];
    unsigned inb = 0;  // bit k: step k stayed in the box and its cell is inside the mask
    const int first = steps;
    P[0] = p;
#pragma unroll
    for (int k = 0; k < LOOKAHEAD; ++k) {
      if (!done && steps >= limit) done = true;
      if (!done) {
        ++steps;
        float3 q;
        float dt;
        grid_step<FAST>(P[k], d, r, s, q, dt);
        t = __fadd_rn(t, dt);
        if (outside_closed3(q, a.n3)) {
          done = true;
          left = true;
        } else {
          P[k + 1] = q;
          T[k] = t;
          const long long idx = cell_index3(P[k], q, a.mask_scale, a.mx, a.my);
          const bool in_mask = idx >= 0 && idx < a.cells;
          // the address is clamped rather than the loaded value selected, so
          // nothing reads the byte before all LOOKAHEAD loads are in flight
          occ[k] = __ldg(a.mask + (in_mask ? idx : 0));
          inb |= (in_mask ? 1u : 0u) << k;
        }
      }
    }
#pragma unroll
    for (int k = 0; k < LOOKAHEAD; ++k) {
      if (((inb >> k) & 1u) && occ[k] != 0) {
        last = first + k + 1;
        if (MODE == WALK_PADDED && count < a.max_n) {
          float* rr = row + 6 * count;
          rr[0] = P[k].x;
          rr[1] = P[k].y;
          rr[2] = P[k].z;
          rr[3] = P[k + 1].x;
          rr[4] = P[k + 1].y;
          rr[5] = P[k + 1].z;
          trow[count] = __fmul_rn(T[k], a.voxel_size);
        }
        if ((MODE == WALK_SEGMENTS || MODE == WALK_SLOTS) && count < cap)
          w.put(a, b, base + count, count + 1 < cap, P[k], P[k + 1], __fmul_rn(T[k], a.voxel_size));
        ++count;
      }
    }
    p = P[LOOKAHEAD];  // only read again when all LOOKAHEAD steps stayed inside
  }
  if (!left && steps >= step_cap) note_cap_hit();
  if (MODE == WALK_SEGMENTS || MODE == WALK_SLOTS) w.flush(a, b);
  if (MODE == WALK_COUNT && a.last_step) a.last_step[b] = last;
  return count;
}

// K steps of lookahead: 16 for small batches (one warp per SM: registers are
// plentiful and the occupancy-load latency is what is left), 8 otherwise
// (the walk is issue-bound once several warps share a scheduler).
template <int MODE, int K = 8>
__global__ void __launch_bounds__(256) masked_walk_kernel(const WalkArgs a) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = b < a.batch;
  int count = 0;
  if (live) {
    const float3 d = load3(a.v, b);
    float3 p = ray_origin_voxel3(a.o, b, a.o3, a.voxel_size);
    float t;
    if (dir_ok(d) && box_entry3(p, d, a.n3, t))
      count = (a.fast && recip_ok(d)) ? masked_walk<MODE, true, K>(a, b, p, d, t)
                                      : masked_walk<MODE, false, K>(a, b, p, d, t);
    else if (MODE == WALK_COUNT && a.last_step)
      a.last_step[b] = 0;
    if (MODE != WALK_SEGMENTS) a.num[b] = count;
  }
  if (MODE != WALK_SEGMENTS) warp_max_atomic(a.max_count, count, live);
}

// Masked-walk emission for large batches, warp-staged.  The 32 rays of a
// warp own separate CSR ranges, so each lane writing its own segments
// scatters 32 stores per instruction across the output.  Here every lane
// stages its segments in shared memory (16 slots: at least two lookahead
// batches between flushes), and when any lane could overflow in the next
// batch, or the warp finishes, the warp writes each lane's run with
// consecutive stores (the run of lane l is contiguous: seg[g_l .. g_l + n_l)).
// Same values, same places as the per-lane writer; the walk arithmetic is the
// same masked walk.  Blocks of one warp: the slots cost 512 B per lane, and
// smaller blocks measured faster (800x800 frame: 2.1 ms, against 2.4 ms with
// two warps per block, 3.3 ms with 8 slots and 4 warps, 3.5 ms per-lane).
constexpr int STAGE_THREADS = 32;
constexpr int STAGE_SLOTS = 16;

__device__ __forceinline__ void grid_step_sel(const float3 a, const float3 d, const float3 r, const float3 s, bool fast,
                                              float3& b, float& dt) {
  if (fast)
    grid_step<true>(a, d, r, s, b, dt);
  else
    grid_step<false>(a, d, r, s, b, dt);
}

__global__ void __launch_bounds__(STAGE_THREADS) masked_emit_staged_kernel(const WalkArgs a) {
  constexpr int K = 8;  // lookahead steps per batch
  __shared__ __align__(16) float stage[STAGE_THREADS * STAGE_SLOTS * 8];  // (6 coords, t, pad) per slot
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const int warp0 = threadIdx.x - lane;  // first thread of this warp in the block
  float* mine = stage + threadIdx.x * STAGE_SLOTS * 8;
  bool done = true, fast = false;
  float3 p = make_float3(0.f, 0.f, 0.f), d = p, r = p, sg = p;
  float t = 0.f;
  int64_t base = 0, cap = 0;
  int count = 0;
  if (b < a.batch) {
    d = load3(a.v, b);
    p = ray_origin_voxel3(a.o, b, a.o3, a.voxel_size);
    if (dir_ok(d) && box_entry3(p, d, a.n3, t)) {
      done = false;
      fast = a.fast && recip_ok(d);
      r = fast ? recip3(d) : d;
      sg = signs(d);
      base = a.offsets[b];
      cap = a.offsets[b + 1] - base;
    }
  }
  int nb = 0;         // staged segments of this lane
  int64_t g = base;   // global index of the first staged one
  int steps = 0;      // walk steps taken; nothing occupied lies beyond `limit`
  const int step_cap = walk_cap(a.n3.x, a.n3.y, a.n3.z);
  const int limit = min((!done && a.stop_step) ? a.stop_step[b] : 0x7fffffff, step_cap);
  bool left = false;  // the walk left the grid
  while (__any_sync(0xffffffffu, !done) || __any_sync(0xffffffffu, nb > 0)) {
    if (!done) {
      float3 P[K + 1];
      float T[K];
      uint8_t occ[K];
      unsigned inb = 0;
      P[0] = p;
#pragma unroll
      for (int k = 0; k < K; ++k) {
        if (!done && steps >= limit) done = true;
        if (!done) {
          ++steps;
          float3 q;
          float dt;
          grid_step_sel(P[k], d, r, sg, fast, q, dt);
          t = __fadd_rn(t, dt);
          if (outside_closed3(q, a.n3)) {
            done = true;
            left = true;
          } else {
            P[k + 1] = q;
            T[k] = t;
            const long long idx = cell_index3(P[k], q, a.mask_scale, a.mx, a.my);
            const bool in_mask = idx >= 0 && idx < a.cells;
            occ[k] = __ldg(a.mask + (in_mask ? idx : 0));
            inb |= (in_mask ? 1u : 0u) << k;
          }
        }
      }
#pragma unroll
      for (int k = 0; k < K; ++k) {
        if (((inb >> k) & 1u) && occ[k] != 0) {
          if (count < cap) {
            float4* slot = reinterpret_cast<float4*>(mine + nb * 8);
            slot[0] = make_float4(P[k].x, P[k].y, P[k].z, P[k + 1].x);
            slot[1] = make_float4(P[k + 1].y, P[k + 1].z, __fmul_rn(T[k], a.voxel_size), 0.f);
            ++nb;
          }
          ++count;
        }
      }
      p = P[K];
    }
    // flush when a lane could overflow in the next batch, or when the warp is finishing
    if (!(__any_sync(0xffffffffu, nb > STAGE_SLOTS - K) || !__any_sync(0xffffffffu, !done))) continue;
    __syncwarp();
    unsigned pending = __ballot_sync(0xffffffffu, nb > 0);
    while (pending) {
      const int l = __ffs(pending) - 1;
      pending &= pending - 1;
      const int n = __shfl_sync(0xffffffffu, nb, l);
      const long long gl = (long long)(((unsigned long long)(unsigned)__shfl_sync(0xffffffffu, (int)(g >> 32), l) << 32) |
                                       (unsigned)__shfl_sync(0xffffffffu, (int)(g & 0xffffffffu), l));
      const float* src = stage + (warp0 + l) * STAGE_SLOTS * 8;
      for (int w = lane; w < n * 6; w += 32) {
        const int k = w / 6;
        a.seg[gl * 6 + w] = src[k * 8 + (w - k * 6)];
      }
      if (lane < n) {
        if (a.seg_t) a.seg_t[gl + lane] = src[lane * 8 + 6];
        if (a.seg_ray) a.seg_ray[gl + lane] = blockIdx.x * blockDim.x + warp0 + l;
      }
    }
    g += nb;
    nb = 0;
    __syncwarp();
  }
  if (b < a.batch && steps > 0 && !left && steps >= step_cap) note_cap_hit();
}

// Slots -> CSR: row k of ray b moves from b * slot + k to offsets[b] + k.
__global__ void __launch_bounds__(256) compact_slots_kernel(int batch, long long slot, const int64_t* __restrict__ offsets,
                                                            const float* __restrict__ sseg,
                                                            const float* __restrict__ st, float* __restrict__ seg,
                                                            float* __restrict__ t, int* __restrict__ ray) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long b = i / slot, k = i - b * slot;
  if (b >= batch) return;
  const long long beg = offsets[b];
  if (k >= offsets[b + 1] - beg) return;
  const long long src = i, dst = beg + k;
  const float2* s2 = reinterpret_cast<const float2*>(sseg + src * 6);
  float2* d2 = reinterpret_cast<float2*>(seg + dst * 6);
  d2[0] = s2[0];
  d2[1] = s2[1];
  d2[2] = s2[2];
  if (t) t[dst] = st[src];
  if (ray) ray[dst] = (int)b;
}

// Octree first hit.  Reference ray_march.cu:33-148, generalised from the
// N in {128, 256} templates to any N that is a multiple of 64.
template <bool FAST>
__device__ __forceinline__ void octree_descend(float* slot, uint8_t* finish, int b, float3 p, const float3 d,
                                               const uint8_t* __restrict__ oct, int N, long long oct_cells) {
  const float3 s = signs(d);
  const float3 r = FAST ? recip3(d) : d;
  int m = N / 64;
  long long off = 0;
  float3 last = p;
  // the levels walk fewer than 3 (N/64 + N/16 + N/4) + 9 <= N + 9 steps in all
  const int cap = walk_cap((float)N, 0.f, 0.f) + 6;
  int steps = 0;
  while (m < N) {
    if (steps++ == cap) {
      note_cap_hit();
      slot[0] = -1.f;
      finish[b] = 1;
      return;
    }
    last = p;
    float3 q;
    float dt;
    grid_step<FAST>(last, d, r, s, q, dt);
    if (outside_closed(q, (float)m)) {
      slot[0] = -1.f;
      finish[b] = 1;
      return;
    }
    const long long idx = off + cell_index1(last, q, m);
    if (occupied(oct, idx, oct_cells)) {
      off += (long long)m * m * m;
      last = make_float3(__fmul_rn(last.x, 4.f), __fmul_rn(last.y, 4.f), __fmul_rn(last.z, 4.f));
      p = last;
      m *= 4;
    } else {
      p = q;
    }
  }
  slot[0] = last.x;
  slot[1] = last.y;
  slot[2] = last.z;
}

__global__ void __launch_bounds__(256) aabb_kernel(int batch, float* __restrict__ coords,
                                                   const float* __restrict__ v,
                                                   const float* __restrict__ center,
                                                   uint8_t* __restrict__ finish,
                                                   float* __restrict__ rgba,
                                                   const uint8_t* __restrict__ oct, int N,
                                                   long long oct_cells) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= batch) return;
  float* slot = coords + (long long)batch * 6 * 7 + (long long)b * 6 + 3;
  reinterpret_cast<float4*>(rgba)[b] = make_float4(0.f, 0.f, 0.f, 1.f);
  finish[b] = 0;
  const float3 d = load3(v, b);
  float3 p = make_float3(__ldg(center + 0), __ldg(center + 1), __ldg(center + 2));
  float t;
  if (!dir_ok(d) || !box_entry(p, d, (float)N, t)) {
    slot[0] = -1.f;
    finish[b] = 1;
    return;
  }
  p = make_float3(__fmul_rn(p.x, 0.015625f), __fmul_rn(p.y, 0.015625f), __fmul_rn(p.z, 0.015625f));
  if (N < (1 << 22) && recip_ok(d))
    octree_descend<true>(slot, finish, b, p, d, oct, N, oct_cells);
  else
    octree_descend<false>(slot, finish, b, p, d, oct, N, oct_cells);
}

// Next 8 occupied voxels.  Reference ray_march.cu:159-229.  The reference
// leaves its grid-stride loop when an unfinished ray has no resume point
// (x < 0), a state that aabb_intersect + mlp_eval never produce; here such a
// ray is skipped on its own so the result does not depend on the launch shape.
template <bool FAST>
__device__ __forceinline__ void march8(float* __restrict__ coords, long long stride, int b, float3 last,
                                       const float3 d, const uint8_t* __restrict__ mask, int N) {
  const float3 s = signs(d);
  const float3 r = FAST ? recip3(d) : d;
  const float n = (float)N;
  const long long cells = (long long)N * N * N;
  const int cap = walk_cap(n, n, n);
  int hits = 0, steps = 0;
  while (hits < 8) {
    if (steps++ == cap) {
      note_cap_hit();
      coords[hits * stride + (long long)b * 6] = -1.f;
      break;
    }
    float3 q;
    float dt;
    grid_step<FAST>(last, d, r, s, q, dt);
    if (outside_open(q, n)) {
      coords[hits * stride + (long long)b * 6] = -1.f;
      break;
    }
    if (occupied(mask, cell_index1(last, q, N), cells)) {
      float2* rr = reinterpret_cast<float2*>(coords + hits * stride + (long long)b * 6);
      rr[0] = make_float2(last.x, last.y);
      rr[1] = make_float2(last.z, q.x);
      rr[2] = make_float2(q.y, q.z);
      ++hits;
    }
    last = q;
  }
}

__global__ void __launch_bounds__(256) march_kernel(int batch, float* __restrict__ coords,
                                                    const float* __restrict__ v,
                                                    const uint8_t* __restrict__ mask,
                                                    const uint8_t* __restrict__ finish, int N) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= batch || finish[b]) return;
  const long long stride = (long long)batch * 6;
  const float* rs = coords + 7 * stride + (long long)b * 6 + 3;
  float3 last = make_float3(rs[0], rs[1], rs[2]);
  coords[(long long)b * 6] = -1.f;
  if (last.x < 0.f) return;
  const float3 d = load3(v, b);
  if (!dir_ok(d)) return;  // a miss (aabb_intersect finished such a ray already)
  const float lim = (float)N;  // a resume point from outside the grid takes the __fdiv_rn form
  if (N < (1 << 22) && recip_ok(d) && fabsf(last.x) <= lim && fabsf(last.y) <= lim && fabsf(last.z) <= lim)
    march8<true>(coords, stride, b, last, d, mask, N);
  else
    march8<false>(coords, stride, b, last, d, mask, N);
}

// Pinhole camera rays (utils/dataset/ray_utils.py:5-55): pixel (i, j) looks
// along ((i + 0.5 - W/2) / focal, -(j + 0.5 - H/2) / focal, -1), rotated by
// the camera-to-world matrix and normalised; the origin is its translation.
struct Camera {
  float r[9];  // rotation, row-major (world = R * camera)
  float t[3];
  float focal;
  int H, W;
  long long first, count;  // pixel range [first, first + count) of the H x W image
};

__global__ void __launch_bounds__(256) camera_rays_kernel(const Camera c, float* __restrict__ o, float* __restrict__ d) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;  // output row
  if (p >= c.count) return;
  const long long px = c.first + p;
  const int j = (int)(px / c.W), i = (int)(px - (long long)j * c.W);
  const float x = __fdiv_rn(__fsub_rn((float)i + 0.5f, 0.5f * (float)c.W), c.focal);
  const float y = -__fdiv_rn(__fsub_rn((float)j + 0.5f, 0.5f * (float)c.H), c.focal);
  float w[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) w[k] = fmaf(c.r[3 * k], x, fmaf(c.r[3 * k + 1], y, -c.r[3 * k + 2]));
  const float n = sqrtf(fmaf(w[0], w[0], fmaf(w[1], w[1], w[2] * w[2])));
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    d[3 * p + k] = __fdiv_rn(w[k], n);
    o[3 * p + k] = c.t[k];
  }
}

__global__ void pair_counts_kernel(int batch, const int* __restrict__ num, int* __restrict__ out) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < batch) out[b] = max(num[b] - 1, 0);
}

// ---- exclusive scan: int32 counts -> int64 offsets --------------------------

__device__ __forceinline__ long long block_exclusive_scan(long long x, long long* smem, long long* total) {
  // warp inclusive scan, then scan of warp totals
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  long long incl = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) smem[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    long long w = lane < (SCAN_THREADS / 32) ? smem[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < SCAN_THREADS / 32) smem[lane] = w;  // inclusive warp-total prefix
  }
  __syncthreads();
  const long long warp_prefix = warp > 0 ? smem[warp - 1] : 0;
  *total = smem[SCAN_THREADS / 32 - 1];
  __syncthreads();
  return warp_prefix + incl - x;
}

__global__ void __launch_bounds__(SCAN_THREADS) scan_tile_sums(const int* __restrict__ in, long long n,
                                                               long long* __restrict__ tile_sum) {
  __shared__ long long smem[32];
  const long long base = (long long)blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
  long long s = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i)
    if (base + i < n) s += in[base + i];
  long long total;
  block_exclusive_scan(s, smem, &total);
  if (threadIdx.x == 0) tile_sum[blockIdx.x] = total;
}

// Single block: exclusive scan of the tile sums in place.
__global__ void __launch_bounds__(SCAN_THREADS) scan_tile_prefix(long long* __restrict__ tile_sum, long long tiles) {
  __shared__ long long smem[32];
  long long carry = 0;
  for (long long start = 0; start < tiles; start += SCAN_THREADS) {
    const long long i = start + threadIdx.x;
    const long long x = i < tiles ? tile_sum[i] : 0;
    long long total;
    const long long ex = block_exclusive_scan(x, smem, &total);
    if (i < tiles) tile_sum[i] = carry + ex;
    carry += total;
  }
}

__global__ void __launch_bounds__(SCAN_THREADS) scan_tiles(const int* __restrict__ in, long long n,
                                                           const long long* __restrict__ tile_prefix,
                                                           int64_t* __restrict__ out) {
  __shared__ long long smem[32];
  const long long base = (long long)blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
  int vals[SCAN_ITEMS];
  long long s = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    vals[i] = base + i < n ? in[base + i] : 0;
    s += vals[i];
  }
  long long total;
  long long run = tile_prefix[blockIdx.x] + block_exclusive_scan(s, smem, &total);
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    if (base + i < n) out[base + i] = run;
    run += vals[i];
  }
  if (base < n && base + SCAN_ITEMS >= n) out[n] = run;  // thread owning the last element
}

}  // namespace dv

using namespace dv;

long long realtime_walk_cap_hits(int reset);  // realtime.cu

// int(voxel_num * mask_scale) with the product rounded to float first, as the
// reference computes it on the device (ray_voxel_intersect.cu:268).
static int cells_per_side(float n, float scale) {
  volatile float prod = n * scale;
  return (int)prod;
}

// Threads per block of a walk launch.  One thread walks one ray and the walk
// is a long dependent chain, so a small batch runs faster spread thinly: with
// fewer rays than 8 warps per SM, blocks of one warp put each warp on its own
// SM instead of several warps sharing a scheduler.
static int walk_block(int batch) {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  return batch < sms * 256 ? 32 : 256;
}

#define DV_COUNT_LAUNCH(batch, stream, args)                                                      \
  do {                                                                                              \
    const int bs__ = walk_block(batch);                                                             \
    if (bs__ == 32)                                                                                 \
      masked_walk_kernel<WALK_COUNT, 16><<<ceil_div((batch), bs__), bs__, 0, (cudaStream_t)(stream)>>>(args); \
    else                                                                                            \
      masked_walk_kernel<WALK_COUNT, 8><<<ceil_div((batch), bs__), bs__, 0, (cudaStream_t)(stream)>>>(args);  \
  } while (0)

#define DV_WALK_LAUNCH(kernel, batch, stream, args)                              \
  do {                                                                             \
    const int bs__ = walk_block(batch);                                            \
    kernel<<<ceil_div((batch), bs__), bs__, 0, (cudaStream_t)(stream)>>>(args);   \
  } while (0)

static bool aligned_to(const void* p, uintptr_t n) { return ((uintptr_t)p % n) == 0; }

// The segment writers store seg with 16-byte (masked) or 8-byte (dense)
// vector stores and seg_t / seg_ray in 8-byte pairs.
static bool segment_buffers_aligned(const float* seg, const float* seg_t, const int* seg_ray, uintptr_t seg_align) {
  return aligned_to(seg, seg_align) && aligned_to(seg_t, 8) && aligned_to(seg_ray, 8);
}

static WalkArgs walk_args(int batch, float xyzmin, float n, float vs, float mask_scale,
                          const float* o, const float* v, const uint8_t* mask) {
  WalkArgs a{};
  a.batch = batch;
  a.xyzmin = xyzmin;
  a.n = n;
  a.o3 = make_float3(xyzmin, xyzmin, xyzmin);
  a.n3 = make_float3(n, n, n);
  a.voxel_size = vs;
  a.mask_scale = mask_scale;
  a.m = cells_per_side(n, mask_scale);
  a.mx = a.my = a.m;
  a.cells = (long long)a.m * a.m * a.m;
  a.fast = n < 4194304.f;
  a.o = o;
  a.v = v;
  a.mask = mask;
  return a;
}

extern "C" {

int dv_ray_voxel_intersect(int batch_size, int max_n, float xyzmin, float xyzmax, float voxel_num,
                           float voxel_size, const float* o, const float* v, float* intersection,
                           int* intersect_num, float* tns, int* max_count, void* stream) {
  (void)xyzmax;  // unused by the reference kernel as well
  DV_CHECK(batch_size >= 0 && max_n >= 0, DV_ERR_ARG);
  if (batch_size == 0) return DV_OK;
  DV_CHECK(o && v && intersect_num && (max_n == 0 || (intersection && tns)), DV_ERR_ARG);
  WalkArgs a = walk_args(batch_size, xyzmin, voxel_num, voxel_size, 1.f, o, v, nullptr);
  a.max_n = max_n;
  a.inter = intersection;
  a.num = intersect_num;
  a.tns = tns;
  a.max_count = max_count;
  DV_WALK_LAUNCH(dense_walk_kernel<WALK_PADDED>, batch_size, stream, a);
  DV_TRY_LAUNCH();
  return DV_OK;
}

int dv_ray_voxel_count(int batch_size, float xyzmin, float voxel_num, float voxel_size,
                       const float* o, const float* v, int* intersect_num, int* max_count,
                       void* stream) {
  DV_CHECK(batch_size >= 0, DV_ERR_ARG);
  if (batch_size == 0) return DV_OK;
  DV_CHECK(o && v && intersect_num, DV_ERR_ARG);
  WalkArgs a = walk_args(batch_size, xyzmin, voxel_num, voxel_size, 1.f, o, v, nullptr);
  a.num = intersect_num;
  a.max_count = max_count;
  DV_WALK_LAUNCH(dense_walk_kernel<WALK_COUNT>, batch_size, stream, a);
  DV_TRY_LAUNCH();
  return DV_OK;
}

int dv_masked_intersect(int batch_size, int max_n, float xyzmin, float xyzmax, float voxel_num,
                        float voxel_size, float mask_scale, const float* o, const float* v,
                        const uint8_t* mask, float* intersection, int* intersect_num, float* tns,
                        int* max_count, void* stream) {
  (void)xyzmax;
  DV_CHECK(batch_size >= 0 && max_n >= 0, DV_ERR_ARG);
  if (batch_size == 0) return DV_OK;
  DV_CHECK(o && v && mask && intersect_num && (max_n == 0 || (intersection && tns)), DV_ERR_ARG);
  WalkArgs a = walk_args(batch_size, xyzmin, voxel_num, voxel_size, mask_scale, o, v, mask);
  a.max_n = max_n;
  a.inter = intersection;
  a.num = intersect_num;
  a.tns = tns;
  a.max_count = max_count;
  DV_WALK_LAUNCH(masked_walk_kernel<WALK_PADDED>, batch_size, stream, a);
  DV_TRY_LAUNCH();
  return DV_OK;
}

int dv_masked_count(int batch_size, float xyzmin, float voxel_num, float voxel_size,
                    float mask_scale, const float* o, const float* v, const uint8_t* mask,
                    int* intersect_num, int* max_count, int* last_step, void* stream) {
  DV_CHECK(batch_size >= 0, DV_ERR_ARG);
  if (batch_size == 0) return DV_OK;
  DV_CHECK(o && v && mask && intersect_num, DV_ERR_ARG);
  WalkArgs a = walk_args(batch_size, xyzmin, voxel_num, voxel_size, mask_scale, o, v, mask);
  a.num = intersect_num;
  a.max_count = max_count;
  a.last_step = last_step;
  DV_COUNT_LAUNCH(batch_size, stream, a);
  DV_TRY_LAUNCH();
  return DV_OK;
}

int dv_masked_segments(int batch_size, float xyzmin, float voxel_num, float voxel_size,
                       float mask_scale, const float* o, const float* v, const uint8_t* mask,
                       const int64_t* offsets, float* seg, float* seg_t, int* seg_ray,
                       const int* stop_step, void* stream) {
  DV_CHECK(batch_size >= 0, DV_ERR_ARG);
  if (batch_size == 0) return DV_OK;
  DV_CHECK(o && v && mask && offsets && seg, DV_ERR_ARG);
  DV_CHECK(segment_buffers_aligned(seg, seg_t, seg_ray, 16), DV_ERR_ARG);
  WalkArgs a = walk_args(batch_size, xyzmin, voxel_num, voxel_size, mask_scale, o, v, mask);
  a.offsets = offsets;
  a.seg = seg;
  a.seg_t = seg_t;
  a.seg_ray = seg_ray;
  a.stop_step = stop_step;
  if (walk_block(batch_size) == 256)
    masked_emit_staged_kernel<<<ceil_div(batch_size, STAGE_THREADS), STAGE_THREADS, 0, (cudaStream_t)stream>>>(a);
  else
    DV_WALK_LAUNCH(masked_walk_kernel<WALK_SEGMENTS>, batch_size, stream, a);
  DV_TRY_LAUNCH();
  return DV_OK;
}

int dv_masked_segments_slots(int batch_size, float xyzmin, float voxel_num, float voxel_size, float mask_scale,
                             const float* o, const float* v, const uint8_t* mask, long long slot, float* seg_slots,
                             float* t_slots, int* intersect_num, int* max_count, void* stream) {
  DV_CHECK(batch_size >= 0, DV_ERR_ARG);
  if (batch_size == 0) return DV_OK;
  DV_CHECK(o && v && mask && seg_slots && t_slots && intersect_num, DV_ERR_ARG);
  DV_CHECK(slot >= (long long)(3.0f * voxel_num) + 3, DV_ERR_ARG);  // no ray crosses more planes
  DV_CHECK(segment_buffers_aligned(seg_slots, t_slots, nullptr, 16), DV_ERR_ARG);
  WalkArgs a = walk_args(batch_size, xyzmin, voxel_num, voxel_size, mask_scale, o, v, mask);
  a.slot = slot;
  a.seg = seg_slots;
  a.seg_t = t_slots;
  a.num = intersect_num;
  a.max_count = max_count;
  DV_WALK_LAUNCH(masked_walk_kernel<WALK_SLOTS>, batch_size, stream, a);
  DV_TRY_LAUNCH();
  return DV_OK;
}

int dv_compact_slots(int batch_size, long long slot, const int64_t* offsets, const float* seg_slots,
                     const float* t_slots, float* seg, float* seg_t, int* seg_ray, void* stream) {
  DV_CHECK(batch_size >= 0 && slot > 0, DV_ERR_ARG);
  if (batch_size == 0) return DV_OK;
  DV_CHECK(offsets && seg_slots && t_slots && seg, DV_ERR_ARG);
  DV_CHECK(aligned_to(seg_slots, 8) && aligned_to(seg, 8), DV_ERR_ARG);
  compact_slots_kernel<<<ceil_div((long long)batch_size * slot, 256), 256, 0, (cudaStream_t)stream>>>(
      batch_size, slot, offsets, seg_slots, t_slots, seg, seg_t, seg_ray);
  DV_TRY_LAUNCH();
  return DV_OK;
}

int dv_dense_segments(int batch_size, float xyzmin, float voxel_num, float voxel_size,
                      const float* o, const float* v, const int64_t* offsets, float* seg,
                      float* seg_t, int* seg_ray, void* stream) {
  DV_CHECK(batch_size >= 0, DV_ERR_ARG);
  if (batch_size == 0) return DV_OK;
  DV_CHECK(o && v && offsets && seg, DV_ERR_ARG);
  DV_CHECK(segment_buffers_aligned(seg, seg_t, seg_ray, 8), DV_ERR_ARG);
  WalkArgs a = walk_args(batch_size, xyzmin, voxel_num, voxel_size, 1.f, o, v, nullptr);
  a.offsets = offsets;
  a.seg = seg;
  a.seg_t = seg_t;
  a.seg_ray = seg_ray;
  DV_WALK_LAUNCH(dense_walk_kernel<WALK_SEGMENTS>, batch_size, stream, a);
  DV_TRY_LAUNCH();
  return DV_OK;
}

int dv_dense_pair_counts(int batch_size, const int* intersect_num, int* seg_count, void* stream) {
  DV_CHECK(batch_size >= 0, DV_ERR_ARG);
  if (batch_size == 0) return DV_OK;
  DV_CHECK(intersect_num && seg_count, DV_ERR_ARG);
  pair_counts_kernel<<<ceil_div(batch_size, 256), 256, 0, (cudaStream_t)stream>>>(batch_size, intersect_num, seg_count);
  DV_TRY_LAUNCH();
  return DV_OK;
}

// Per-axis grids: origin xyzmin[3] (world), extents dims[3] = (nx, ny, nz)
// voxels, occupancy [nz][ny][nx] bytes (mask scale 1).
static WalkArgs walk_args_grid(int batch, const float* xyzmin, const int* dims, float vs, const float* o,
                               const float* v, const uint8_t* mask) {
  WalkArgs a{};
  a.batch = batch;
  a.o3 = make_float3(xyzmin[0], xyzmin[1], xyzmin[2]);
  a.n3 = make_float3((float)dims[0], (float)dims[1], (float)dims[2]);
  a.voxel_size = vs;
  a.mask_scale = 1.f;
  a.mx = dims[0];
  a.my = dims[1];
  a.cells = (long long)dims[0] * dims[1] * dims[2];
  a.fast = dims[0] < (1 << 22) && dims[1] < (1 << 22) && dims[2] < (1 << 22);
  a.o = o;
  a.v = v;
  a.mask = mask;
  return a;
}

int dv_camera_rays(int H, int W, float focal, const float* c2w, long long first_pixel, long long n_pixels,
                   float* rays_o, float* rays_d, void* stream) {
  DV_CHECK(H >= 0 && W >= 0 && c2w && first_pixel >= 0 && n_pixels >= 0, DV_ERR_ARG);
  DV_CHECK(first_pixel + n_pixels <= (long long)H * W, DV_ERR_ARG);
  if (n_pixels == 0) return DV_OK;
  DV_CHECK(rays_o && rays_d, DV_ERR_ARG);
  Camera c{};
  for (int k = 0; k < 3; ++k) {
    for (int l = 0; l < 3; ++l) c.r[3 * k + l] = c2w[4 * k + l];
    c.t[k] = c2w[4 * k + 3];
  }
  c.focal = focal;
  c.H = H;
  c.W = W;
  c.first = first_pixel;
  c.count = n_pixels;
  camera_rays_kernel<<<ceil_div(n_pixels, 256), 256, 0, (cudaStream_t)stream>>>(c, rays_o, rays_d);
  DV_TRY_LAUNCH();
  return DV_OK;
}

int dv_masked_count_grid(int batch_size, const float* xyzmin, const int* dims, float voxel_size, const float* o,
                         const float* v, const uint8_t* mask, int* intersect_num, int* max_count, int* last_step,
                         void* stream) {
  DV_CHECK(batch_size >= 0 && xyzmin && dims && dims[0] > 0 && dims[1] > 0 && dims[2] > 0, DV_ERR_ARG);
  if (batch_size == 0) return DV_OK;
  DV_CHECK(o && v && mask && intersect_num, DV_ERR_ARG);
  WalkArgs a = walk_args_grid(batch_size, xyzmin, dims, voxel_size, o, v, mask);
  a.num = intersect_num;
  a.max_count = max_count;
  a.last_step = last_step;
  DV_COUNT_LAUNCH(batch_size, stream, a);
  DV_TRY_LAUNCH();
  return DV_OK;
}

int dv_masked_segments_grid(int batch_size, const float* xyzmin, const int* dims, float voxel_size, const float* o,
                            const float* v, const uint8_t* mask, const int64_t* offsets, float* seg, float* seg_t,
                            int* seg_ray, const int* stop_step, void* stream) {
  DV_CHECK(batch_size >= 0 && xyzmin && dims && dims[0] > 0 && dims[1] > 0 && dims[2] > 0, DV_ERR_ARG);
  if (batch_size == 0) return DV_OK;
  DV_CHECK(o && v && mask && offsets && seg, DV_ERR_ARG);
  DV_CHECK(segment_buffers_aligned(seg, seg_t, seg_ray, 16), DV_ERR_ARG);
  WalkArgs a = walk_args_grid(batch_size, xyzmin, dims, voxel_size, o, v, mask);
  a.offsets = offsets;
  a.seg = seg;
  a.seg_t = seg_t;
  a.seg_ray = seg_ray;
  a.stop_step = stop_step;
  if (walk_block(batch_size) == 256)
    masked_emit_staged_kernel<<<ceil_div(batch_size, STAGE_THREADS), STAGE_THREADS, 0, (cudaStream_t)stream>>>(a);
  else
    DV_WALK_LAUNCH(masked_walk_kernel<WALK_SEGMENTS>, batch_size, stream, a);
  DV_TRY_LAUNCH();
  return DV_OK;
}

long long dv_walk_cap_hits(int reset) {
  unsigned long long v = 0, w = 0;
  if (cudaMemcpyFromSymbol(&v, g_walk_cap_hits, sizeof(v)) != cudaSuccess) return -1;
  const long long rt = realtime_walk_cap_hits(reset);
  if (rt < 0) return -1;
  if (reset && cudaMemcpyToSymbol(g_walk_cap_hits, &w, sizeof(w)) != cudaSuccess) return -1;
  return (long long)v + rt;
}

long long dv_scan_scratch_bytes(long long n) {
  const long long tiles = n > 0 ? (n + SCAN_TILE - 1) / SCAN_TILE : 1;
  return tiles * (long long)sizeof(long long);
}

int dv_exclusive_scan(const int* counts, long long n, int64_t* offsets, void* scratch, void* stream) {
  DV_CHECK(n >= 0 && offsets, DV_ERR_ARG);
  cudaStream_t st = (cudaStream_t)stream;
  if (n == 0) {
    if (cudaMemsetAsync(offsets, 0, sizeof(int64_t), st) != cudaSuccess) return DV_ERR_CUDA;
    return DV_OK;
  }
  DV_CHECK(counts && scratch, DV_ERR_ARG);
  const long long tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  DV_CHECK(tiles < (1LL << 31), DV_ERR_ARG);
  long long* tile_sum = (long long*)scratch;
  scan_tile_sums<<<(unsigned)tiles, SCAN_THREADS, 0, st>>>(counts, n, tile_sum);
  scan_tile_prefix<<<1, SCAN_THREADS, 0, st>>>(tile_sum, tiles);
  scan_tiles<<<(unsigned)tiles, SCAN_THREADS, 0, st>>>(counts, n, tile_sum, offsets);
  DV_TRY_LAUNCH();
  return DV_OK;
}

int dv_aabb_intersect(int batch_size, float* coords, const float* v, const float* center,
                      uint8_t* finish, float* rgba, const uint8_t* octrees, int voxel_num,
                      void* stream) {
  DV_CHECK(batch_size >= 0 && voxel_num >= 64 && voxel_num % 64 == 0, DV_ERR_ARG);
  if (batch_size == 0) return DV_OK;
  DV_CHECK(coords && v && center && finish && rgba && octrees, DV_ERR_ARG);
  DV_CHECK(((uintptr_t)rgba & 15) == 0, DV_ERR_ARG);
  const long long a = voxel_num / 64, b = voxel_num / 16, c = voxel_num / 4;
  const long long cells = a * a * a + b * b * b + c * c * c;
  aabb_kernel<<<ceil_div(batch_size, 256), 256, 0, (cudaStream_t)stream>>>(
      batch_size, coords, v, center, finish, rgba, octrees, voxel_num, cells);
  DV_TRY_LAUNCH();
  return DV_OK;
}

int dv_ray_march(int batch_size, float* coords, const float* v, const uint8_t* mask,
                 const uint8_t* finish, int voxel_num, void* stream) {
  DV_CHECK(batch_size >= 0 && voxel_num > 0, DV_ERR_ARG);
  if (batch_size == 0) return DV_OK;
  DV_CHECK(coords && v && mask && finish, DV_ERR_ARG);
  DV_CHECK(aligned_to(coords, 8), DV_ERR_ARG);
  march_kernel<<<ceil_div(batch_size, 256), 256, 0, (cudaStream_t)stream>>>(batch_size, coords, v, mask,
                                                                           finish, voxel_num);
  DV_TRY_LAUNCH();
  return DV_OK;
}

}  // extern "C"
