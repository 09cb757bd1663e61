// Shared layout of the real-time decoder's weights (realtime.cu, realtime_tc.cu).
#pragma once
#include "mlp.cuh"

namespace dv {

// Aligned real-time layout (floats), width W, FIRST = 1 for DIVeR32 (bias of
// the pre-multiplied first layer, applied to the integrated feature):
//   [FIRST] b_in [32]
//   L0   bias [W], W^T [32][W]       (weight0: 32 -> W)
//   SIG  w [W], bias, pad -> W+4     (weight1: sigma)
//   L2   bias [W], W^T [W][W], W^T_pe [28][W] (torch PE order, row 27 zero)
//   L3   bias [4], W^T [W][4]        (weight3: W -> 3)
template <int W, int FIRST>
struct RtLayout {
  static constexpr int b_in = 0;
  static constexpr int l0_b = FIRST ? 32 : 0;
  static constexpr int l0_w = l0_b + W;
  static constexpr int sig = l0_w + 32 * W;
  static constexpr int l2_b = sig + W + 4;
  static constexpr int l2_w = l2_b + W;
  static constexpr int l2_pe = l2_w + W * W;
  static constexpr int l3_b = l2_pe + PE_PAD * W;
  static constexpr int l3_w = l3_b + 4;
  static constexpr int size = l3_w + W * 4;
};

// Reference params index of the PE weight of torch PE column k (the reference
// stores per axis [d, sin x4, cos x4]; convert.py:89-92,128-131).
__host__ __device__ inline int pe_ref_row(int k) {
  if (k < 3) return k * 9;
  const int band = (k - 3) / 6, r = (k - 3) % 6, ax = r % 3;
  return ax * 9 + (r < 3 ? 1 + band : 5 + band);
}

}  // namespace dv
