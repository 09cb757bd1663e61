// Shared device helpers for the DIVeR hot-path kernels (sm_103a).
//
// Every floating-point step of the voxel walk is written with explicit
// round-to-nearest intrinsics (__fadd_rn, __fmul_rn, __fdiv_rn, __fmaf_rn) so
// the result does not depend on the compiler's contraction choices.  The walk
// reproduces the reference kernels' arithmetic exactly:
//   utils/ray_voxel_intersection/src/ray_voxel_intersect.cu:53-150 (dense)
//   utils/ray_voxel_intersection/src/ray_voxel_intersect.cu:216-318 (masked)
//   utils/ray_march/src/ray_march.cu:58-145,184-227 (octree + march)
// The reference is compiled with the default -fmad=true, which contracts the
// position update `ori + dir*t` into one fused multiply-add; the products
// `ori*step` and `floor(..)*step` are exact (step is -1, 0 or +1), so writing
// them fused or unfused gives the same bits.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/diver_gb300.h"

namespace dv {

// A direction with a non-finite component, or a zero direction, does not
// advance one grid plane per step (its steps are NaN or -inf, and NaN points
// never test as outside the grid): the walks treat such a ray as a miss.  The
// reference kernels have no such check and never leave their loop on it.
__device__ __forceinline__ bool dir_ok(const float3 d) {
  return isfinite(d.x) && isfinite(d.y) && isfinite(d.z) && (d.x != 0.f || d.y != 0.f || d.z != 0.f);
}

// Step bound of a walk through a box of nx x ny x nz cells.  Every step snaps
// one axis onto its next grid plane (the plane along the direction's sign,
// strictly ahead of the point) and every coordinate moves monotonically, so a
// ray crosses at most n + 1 planes per axis before it leaves: no walk of a ray
// that passes dir_ok takes more steps.  The walks stop there all the same and
// count the stop (note_cap_hit), so that no arithmetic case can keep a thread
// walking.
__host__ __device__ __forceinline__ int walk_cap(float nx, float ny, float nz) { return (int)(nx + ny + nz) + 3; }

// Walks (of this translation unit) that stopped at walk_cap; read by
// dv_walk_cap_hits.
static __device__ unsigned long long g_walk_cap_hits;
__device__ __forceinline__ void note_cap_hit() { atomicAdd(&g_walk_cap_hits, 1ull); }

// Sign of x as -1, 0 or +1 (reference ray_voxel_intersect.cu:9-13).
__device__ __forceinline__ float step_sign(float x) {
  return x > 0.f ? 1.f : (x < 0.f ? -1.f : 0.f);
}

__device__ __forceinline__ float clampf(float v, float lo, float hi) {
  return fmaxf(lo, fminf(v, hi));
}

// Slab test against the box [0, n.x] x [0, n.y] x [0, n.z] (per-axis extents;
// with n.x = n.y = n.z the arithmetic is exactly the cubic test below).
__device__ __forceinline__ bool box_entry3(float3& p, const float3 d, const float3 n, float& t) {
  const bool inside = (p.x >= 0.f) & (p.y >= 0.f) & (p.z >= 0.f) &
                      (p.x <= n.x) & (p.y <= n.y) & (p.z <= n.z);
  if (inside) {
    t = 0.f;
    return true;
  }
  float a = __fdiv_rn(-p.x, d.x), b = __fdiv_rn(__fsub_rn(n.x, p.x), d.x);
  float lo = fminf(a, b), hi = fmaxf(a, b);
  a = __fdiv_rn(-p.y, d.y);
  b = __fdiv_rn(__fsub_rn(n.y, p.y), d.y);
  lo = fmaxf(lo, fminf(a, b));
  hi = fminf(hi, fmaxf(a, b));
  a = __fdiv_rn(-p.z, d.z);
  b = __fdiv_rn(__fsub_rn(n.z, p.z), d.z);
  lo = fmaxf(lo, fminf(a, b));
  hi = fminf(hi, fmaxf(a, b));
  p.x = clampf(__fmaf_rn(d.x, lo, p.x), 0.f, n.x);
  p.y = clampf(__fmaf_rn(d.y, lo, p.y), 0.f, n.y);
  p.z = clampf(__fmaf_rn(d.z, lo, p.z), 0.f, n.z);
  t = lo;
  return !(lo > hi);
}

__device__ __forceinline__ bool outside_closed3(const float3 b, const float3 n) {
  return (b.x < 0.f) | (b.y < 0.f) | (b.z < 0.f) | (b.x > n.x) | (b.y > n.y) | (b.z > n.z);
}

// Linear occupancy index on an mx x my x mz grid (x fastest).
__device__ __forceinline__ long long cell_index3(const float3 a, const float3 b, float scale, int mx, int my) {
  const float cx = __fmul_rn(fminf(__fadd_rn(a.x, 1e-4f), __fadd_rn(b.x, 1e-4f)), scale);
  const float cy = __fmul_rn(fminf(__fadd_rn(a.y, 1e-4f), __fadd_rn(b.y, 1e-4f)), scale);
  const float cz = __fmul_rn(fminf(__fadd_rn(a.z, 1e-4f), __fadd_rn(b.z, 1e-4f)), scale);
  return ((long long)(int)cz * my + (int)cy) * mx + (int)cx;
}

// Slab test of the ray (p, d) against the box [0, n]^3 in voxel units.
// When p lies inside the box it is kept and t = 0.  Otherwise p becomes the
// clamped point p + d*tmin and t = tmin.  Returns false on a miss (tmin > tmax);
// p still holds the clamped point then, which the dense walk records.
// Reference: ray_voxel_intersect.cu:61-100, ray_march.cu:58-88.
__device__ __forceinline__ bool box_entry(float3& p, const float3 d, const float n, float& t) {
  const bool inside = (p.x >= 0.f) & (p.y >= 0.f) & (p.z >= 0.f) &
                      (p.x <= n) & (p.y <= n) & (p.z <= n);
  if (inside) {
    t = 0.f;
    return true;
  }
  float a = __fdiv_rn(-p.x, d.x), b = __fdiv_rn(__fsub_rn(n, p.x), d.x);
  float lo = fminf(a, b), hi = fmaxf(a, b);
  a = __fdiv_rn(-p.y, d.y);
  b = __fdiv_rn(__fsub_rn(n, p.y), d.y);
  lo = fmaxf(lo, fminf(a, b));
  hi = fminf(hi, fmaxf(a, b));
  a = __fdiv_rn(-p.z, d.z);
  b = __fdiv_rn(__fsub_rn(n, p.z), d.z);
  lo = fmaxf(lo, fminf(a, b));
  hi = fminf(hi, fmaxf(a, b));
  p.x = clampf(__fmaf_rn(d.x, lo, p.x), 0.f, n);
  p.y = clampf(__fmaf_rn(d.y, lo, p.y), 0.f, n);
  p.z = clampf(__fmaf_rn(d.z, lo, p.z), 0.f, n);
  t = lo;
  return !(lo > hi);
}

// Quotient x / d rounded to nearest from r = RN(1/d):
//   q = RN(x * r),  e = x - d * q (exact in one FMA),  result = RN(q + e * r).
// By Markstein's theorem (P. W. Markstein, "Computation of elementary
// functions on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1),
// 1990) this is the correctly rounded quotient, the same bits as __fdiv_rn,
// whenever no intermediate overflows or underflows.  The walks divide the
// distance to the next grid plane (|x| between 2^-24 and 2 for points inside
// a grid of fewer than 2^23 voxels per side) by a direction component, so
// recip_ok() admits a direction only when every component has
// 2^-60 <= |d| <= 2^60; other rays take the __fdiv_rn form of the step.
__device__ __forceinline__ float div_by_recip(float x, float d, float r) {
  const float q = __fmul_rn(x, r);
  const float e = __fmaf_rn(-q, d, x);
  return __fmaf_rn(e, r, q);
}

__device__ __forceinline__ bool recip_ok(const float3 d) {
  const float lo = 8.67361738e-19f, hi = 1.15292150e18f;  // 2^-60, 2^60
  const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
  return (ax >= lo) & (ax <= hi) & (ay >= lo) & (ay <= hi) & (az >= lo) & (az <= hi);
}

__device__ __forceinline__ float3 recip3(const float3 d) {
  return make_float3(__frcp_rn(d.x), __frcp_rn(d.y), __frcp_rn(d.z));
}

template <bool FAST>
__device__ __forceinline__ float step_div(float x, float d, float r) {
  if constexpr (FAST) {
    return div_by_recip(x, d, r);
  } else {
    return __fdiv_rn(x, d);
  }
}

// One step of the 3D-DDA: from point a, move along d to the nearest grid
// plane crossing b; dt is the parameter increment.  The coordinate of the
// plane that was hit is snapped onto the plane, with ties resolved x, then y,
// then z.  r = recip3(d) when FAST (unused otherwise).
// Reference: ray_voxel_intersect.cu:119-135.
template <bool FAST>
__device__ __forceinline__ void grid_step(const float3 a, const float3 d, const float3 r, const float3 s,
                                          float3& b, float& dt) {
  const float bx = __fmul_rn(floorf(__fmaf_rn(a.x, s.x, 1.f)), s.x);
  const float by = __fmul_rn(floorf(__fmaf_rn(a.y, s.y, 1.f)), s.y);
  const float bz = __fmul_rn(floorf(__fmaf_rn(a.z, s.z, 1.f)), s.z);
  const float tx = step_div<FAST>(__fsub_rn(bx, a.x), d.x, r.x);
  const float ty = step_div<FAST>(__fsub_rn(by, a.y), d.y, r.y);
  const float tz = step_div<FAST>(__fsub_rn(bz, a.z), d.z, r.z);
  dt = fminf(tx, fminf(ty, tz));
  b.x = __fmaf_rn(d.x, dt, a.x);
  b.y = __fmaf_rn(d.y, dt, a.y);
  b.z = __fmaf_rn(d.z, dt, a.z);
  if (dt == tx) {
    b.x = bx;
  } else if (dt == ty) {
    b.y = by;
  } else {
    b.z = bz;
  }
}

// True when b has left [0, n]^3 (dense and masked walks: a point on the far
// face is still inside).  Reference: ray_voxel_intersect.cu:137-138.
__device__ __forceinline__ bool outside_closed(const float3 b, const float n) {
  return (b.x < 0.f) | (b.y < 0.f) | (b.z < 0.f) | (b.x > n) | (b.y > n) | (b.z > n);
}

// True when b has left [0, n)^3 (real-time march).  Reference: ray_march.cu:203-204.
__device__ __forceinline__ bool outside_open(const float3 b, const float n) {
  return (b.x < 0.f) | (b.y < 0.f) | (b.z < 0.f) | (b.x >= n) | (b.y >= n) | (b.z >= n);
}

// Linear index of the occupancy cell that holds the voxel between a and b,
// on a grid of m cells per side scaled by `scale` from voxel units.
// Reference: ray_voxel_intersect.cu:297-299, ray_march.cu:132-135,211-212.
__device__ __forceinline__ long long cell_index(const float3 a, const float3 b, float scale, int m) {
  const float cx = __fmul_rn(fminf(__fadd_rn(a.x, 1e-4f), __fadd_rn(b.x, 1e-4f)), scale);
  const float cy = __fmul_rn(fminf(__fadd_rn(a.y, 1e-4f), __fadd_rn(b.y, 1e-4f)), scale);
  const float cz = __fmul_rn(fminf(__fadd_rn(a.z, 1e-4f), __fadd_rn(b.z, 1e-4f)), scale);
  return (long long)(int)cz * m * m + (long long)(int)cy * m + (int)cx;
}

// Same index without the scale factor (scale == 1 multiplies exactly).
__device__ __forceinline__ long long cell_index1(const float3 a, const float3 b, int m) {
  const float cx = fminf(__fadd_rn(a.x, 1e-4f), __fadd_rn(b.x, 1e-4f));
  const float cy = fminf(__fadd_rn(a.y, 1e-4f), __fadd_rn(b.y, 1e-4f));
  const float cz = fminf(__fadd_rn(a.z, 1e-4f), __fadd_rn(b.z, 1e-4f));
  return (long long)(int)cz * m * m + (long long)(int)cy * m + (int)cx;
}

// Reads one occupancy byte; an index outside the mask (a degenerate walk
// along the far face) counts as empty instead of reading past the buffer.
__device__ __forceinline__ bool occupied(const uint8_t* __restrict__ mask, long long idx, long long cells) {
  return (idx >= 0 && idx < cells) ? (__ldg(mask + idx) != 0) : false;
}

// Segment count of a decode launch: `cap` (the host count, or the capacity of
// the segment buffers) or, when `dev` is given, the count the device holds
// there (the CSR end offsets[B]) clamped to [0, cap].  Reading it on the
// device lets a launch be recorded in a CUDA graph before the count exists.
__device__ __forceinline__ long long segment_total(long long cap, const int64_t* dev) {
  if (dev == nullptr) return cap;
  const long long v = (long long)*dev;
  return v < 0 ? 0 : (v < cap ? v : cap);
}

__host__ __device__ __forceinline__ unsigned ceil_div(long long a, long long b) {
  return (unsigned)((a + b - 1) / b);
}

}  // namespace dv

// Error helpers used by every C-ABI entry point: a launch failure becomes a
// status code, never a process exit.
#define DV_TRY_LAUNCH()                                   \
  do {                                                    \
    cudaError_t e__ = cudaGetLastError();                 \
    if (e__ != cudaSuccess) return DV_ERR_CUDA;           \
  } while (0)

#define DV_CHECK(cond, code) \
  do {                       \
    if (!(cond)) return (code); \
  } while (0)
