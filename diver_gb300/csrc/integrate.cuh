// Closed-form segment integral of a trilinear feature field (device helpers).
//
// The mean of the trilinear interpolant of the 8 corner vectors along a
// segment P0 -> P1 (local voxel coordinates) is sum_j w_j F_j with the corner
// weights below, the same polynomial as the reference's
//   feature = A*X + sum_d B_d*Y_d + sum_d C_d*Z_d + F000
// (utils/integrator.py:88-111, weights spelled out in
//  utils/mlp_evaluation/src/mlp_eval.cu:83-101).  Weights sum to 1.
// Corner j: bit 0 = +x, bit 1 = +y, bit 2 = +z.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace dv {

struct SegCorner {
  int x, y, z;      // lower corner (pmin)
  int x1, y1, z1;   // upper corner, clamped to the grid
  float w[8];
};

// pmin = min(int(p0 + 1e-4), int(p1 + 1e-4)) per axis (utils/integrator.py:75);
// the upper corner is clamped to n_vert - 1 (:79).  Negative or oversized
// lower corners (never produced by the walks) are clamped into the grid.
__device__ __forceinline__ SegCorner segment_corners(float x0, float y0, float z0, float x1, float y1,
                                                     float z1, int nvx, int nvy, int nvz) {
  SegCorner c;
  c.x = min((int)__fadd_rn(x0, 1e-4f), (int)__fadd_rn(x1, 1e-4f));
  c.y = min((int)__fadd_rn(y0, 1e-4f), (int)__fadd_rn(y1, 1e-4f));
  c.z = min((int)__fadd_rn(z0, 1e-4f), (int)__fadd_rn(z1, 1e-4f));
  const float X0 = x0 - (float)c.x, X1 = x1 - (float)c.x;
  const float Y0 = y0 - (float)c.y, Y1 = y1 - (float)c.y;
  const float Z0 = z0 - (float)c.z, Z1 = z1 - (float)c.z;
  c.x = max(0, min(c.x, nvx - 1));
  c.y = max(0, min(c.y, nvy - 1));
  c.z = max(0, min(c.z, nvz - 1));
  c.x1 = min(c.x + 1, nvx - 1);
  c.y1 = min(c.y + 1, nvy - 1);
  c.z1 = min(c.z + 1, nvz - 1);
  // moments of the local coordinates along the segment
  const float ix = 0.5f * (X0 + X1), iy = 0.5f * (Y0 + Y1), iz = 0.5f * (Z0 + Z1);
  const float ixy = (X0 * Y0 + X1 * Y1) * (1.f / 3.f) + (X0 * Y1 + X1 * Y0) * (1.f / 6.f);
  const float iyz = (Y0 * Z0 + Y1 * Z1) * (1.f / 3.f) + (Y0 * Z1 + Y1 * Z0) * (1.f / 6.f);
  const float ixz = (X0 * Z0 + X1 * Z1) * (1.f / 3.f) + (X0 * Z1 + X1 * Z0) * (1.f / 6.f);
  const float ixyz = (X0 + X1) * (Y0 + Y1) * (Z0 + Z1) * (1.f / 12.f) + (X0 * Y0 * Z0 + X1 * Y1 * Z1) * (1.f / 6.f);
  c.w[7] = ixyz;
  c.w[3] = ixy - ixyz;
  c.w[5] = ixz - ixyz;
  c.w[6] = iyz - ixyz;
  c.w[1] = ix - ixy - ixz + ixyz;
  c.w[2] = iy - ixy - iyz + ixyz;
  c.w[4] = iz - ixz - iyz + ixyz;
  c.w[0] = 1.f - ix - iy - iz + ixy + iyz + ixz - ixyz;
  return c;
}

// Row (corner) offset, in elements / channels, of corner j of a segment.
__device__ __forceinline__ long long corner_row(const SegCorner& c, int j, int nvx, int nvy) {
  const int x = (j & 1) ? c.x1 : c.x;
  const int y = (j & 2) ? c.y1 : c.y;
  const int z = (j & 4) ? c.z1 : c.z;
  return ((long long)z * nvy + y) * nvx + x;
}

__device__ __forceinline__ float4 ldg4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }

__device__ __forceinline__ void fma4(float4& acc, float w, const float4 v) {
  acc.x = fmaf(w, v.x, acc.x);
  acc.y = fmaf(w, v.y, acc.y);
  acc.z = fmaf(w, v.z, acc.z);
  acc.w = fmaf(w, v.w, acc.w);
}

// Integrated features, channels [c4*4, c4*4+4) of one segment.
__device__ __forceinline__ float4 integrate4(const float* __restrict__ grid, const SegCorner& sc, int C, int c4,
                                             int nvx, int nvy) {
  float4 v[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) v[j] = ldg4(grid + corner_row(sc, j, nvx, nvy) * C + c4 * 4);
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int j = 0; j < 8; ++j) fma4(acc, sc.w[j], v[j]);
  return acc;
}

// Vector atomic add of 4 floats (sm_90+ global float4 atomics).
__device__ __forceinline__ void red_add4(float* dst, float4 v) {
  atomicAdd(reinterpret_cast<float4*>(dst), v);
}

// Scatters w_j * g into the 8 corner rows (channels [c4*4, c4*4+4)).
__device__ __forceinline__ void scatter4(float* __restrict__ grad, const SegCorner& sc, int C, int c4, float4 g,
                                         int nvx, int nvy) {
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float w = sc.w[j];
    red_add4(grad + corner_row(sc, j, nvx, nvy) * C + c4 * 4, make_float4(w * g.x, w * g.y, w * g.z, w * g.w));
  }
}

}  // namespace dv
