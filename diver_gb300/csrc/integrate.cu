// Feature integration over segments (forward) and its gradient with respect
// to the corner features (backward), for the reference's `integrate`
// (utils/integrator.py:62-112).
//
// Layout: C/4 consecutive threads own one segment, each a float4 of
// channels, so the 8 corner reads of a segment are C*4-byte contiguous,
// coalesced requests.  The backward scatters w_j * dL/dfeature into the 8
// corner rows with float4 vector atomics (red.global.add.v4.f32).
#include "common.cuh"
#include "integrate.cuh"

namespace dv {

struct IntegrateArgs {
  const float* grid;   // forward: voxels
  float* grad_grid;    // backward: d voxels (accumulated)
  const float* ci;     // entry points, row stride `stride`
  const float* co;     // exit points
  long long stride;
  long long n_seg;
  const float* gin;    // backward: d feature [S][C]
  float* out;          // forward: feature [S][C]
  int nvx, nvy, nvz, C;
  const int64_t* rows; // implicit stage: table row of each segment's 8 corners
};

__global__ void __launch_bounds__(256) integrate_fwd_kernel(const IntegrateArgs a) {
  const int tps = a.C >> 2;
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long s = tid / tps;
  const int c4 = (int)(tid - s * tps);
  if (s >= a.n_seg) return;
  const float* pi = a.ci + s * a.stride;
  const float* po = a.co + s * a.stride;
  const SegCorner sc = segment_corners(__ldg(pi), __ldg(pi + 1), __ldg(pi + 2), __ldg(po), __ldg(po + 1),
                                       __ldg(po + 2), a.nvx, a.nvy, a.nvz);
  const float4 f = integrate4(a.grid, sc, a.C, c4, a.nvx, a.nvy);
  reinterpret_cast<float4*>(a.out + s * a.C)[c4] = f;
}

__global__ void __launch_bounds__(256) integrate_bwd_kernel(const IntegrateArgs a) {
  const int tps = a.C >> 2;
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long s = tid / tps;
  const int c4 = (int)(tid - s * tps);
  if (s >= a.n_seg) return;
  const float* pi = a.ci + s * a.stride;
  const float* po = a.co + s * a.stride;
  const SegCorner sc = segment_corners(__ldg(pi), __ldg(pi + 1), __ldg(pi + 2), __ldg(po), __ldg(po + 1),
                                       __ldg(po + 2), a.nvx, a.nvy, a.nvz);
  const float4 g = ldg4(a.gin + s * a.C + c4 * 4);
  scatter4(a.grad_grid, sc, a.C, c4, g, a.nvx, a.nvy);
}

// ---- implicit stage: features from a table of unique corners -------------
// (utils/integrator.py:3-59).  rows [S][8]: the table row of each segment's
// corner j (bit 0 = +x, bit 1 = +y, bit 2 = +z); the corner weights are those
// of the explicit integral, from the segment's local coordinates.

// rows[s][j] = linear index (z * nv + y) * nv + x of corner j, with the lower
// corner min(int(p0 + 1e-4), int(p1 + 1e-4)) and the upper one clamped to
// nv - 1 (utils/integrator.py:16-28).
__global__ void __launch_bounds__(256) corner_rows_kernel(const float* __restrict__ ci, const float* __restrict__ co,
                                                          long long stride, long long n_seg, int nv,
                                                          int64_t* __restrict__ rows) {
  const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n_seg) return;
  const float* pi = ci + s * stride;
  const float* po = co + s * stride;
  int lo[3], hi[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    lo[k] = min((int)__fadd_rn(__ldg(pi + k), 1e-4f), (int)__fadd_rn(__ldg(po + k), 1e-4f));
    hi[k] = min(lo[k] + 1, nv - 1);
  }
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const long long x = (j & 1) ? hi[0] : lo[0], y = (j & 2) ? hi[1] : lo[1], z = (j & 4) ? hi[2] : lo[2];
    rows[s * 8 + j] = (z * nv + y) * nv + x;
  }
}

__global__ void __launch_bounds__(256) integrate_table_fwd_kernel(const IntegrateArgs a) {
  const int tps = a.C >> 2;
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long s = tid / tps;
  const int c4 = (int)(tid - s * tps);
  if (s >= a.n_seg) return;
  const float* pi = a.ci + s * a.stride;
  const float* po = a.co + s * a.stride;
  const SegCorner sc = segment_corners(__ldg(pi), __ldg(pi + 1), __ldg(pi + 2), __ldg(po), __ldg(po + 1),
                                       __ldg(po + 2), 1 << 30, 1 << 30, 1 << 30);
  const int64_t* r = a.rows + s * 8;
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int j = 0; j < 8; ++j) fma4(acc, sc.w[j], ldg4(a.grid + __ldg(r + j) * a.C + c4 * 4));
  reinterpret_cast<float4*>(a.out + s * a.C)[c4] = acc;
}

__global__ void __launch_bounds__(256) integrate_table_bwd_kernel(const IntegrateArgs a) {
  const int tps = a.C >> 2;
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long s = tid / tps;
  const int c4 = (int)(tid - s * tps);
  if (s >= a.n_seg) return;
  const float* pi = a.ci + s * a.stride;
  const float* po = a.co + s * a.stride;
  const SegCorner sc = segment_corners(__ldg(pi), __ldg(pi + 1), __ldg(pi + 2), __ldg(po), __ldg(po + 1),
                                       __ldg(po + 2), 1 << 30, 1 << 30, 1 << 30);
  const float4 g = ldg4(a.gin + s * a.C + c4 * 4);
  const int64_t* r = a.rows + s * 8;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float w = sc.w[j];
    red_add4(a.grad_grid + __ldg(r + j) * a.C + c4 * 4, make_float4(w * g.x, w * g.y, w * g.z, w * g.w));
  }
}

static int check_common(const IntegrateArgs& a) {
  if (a.n_seg < 0 || a.C <= 0 || (a.C & 3) || a.nvx <= 0 || a.nvy <= 0 || a.nvz <= 0 || a.stride < 3) return DV_ERR_ARG;
  if (a.n_seg > 0 && (!a.ci || !a.co)) return DV_ERR_ARG;
  return DV_OK;
}

// ---- clearing only the gradient rows a step wrote ------------------------
//
// A training step accumulates into the 8 corner rows of each of its segments,
// a small part of a large grid (about 3 M of 17 M rows for 4096 rays through a
// 256^3 grid), so zeroing the whole gradient before every step moves ~5x the
// bytes the step writes.  mark_rows_kernel sets one byte per segment at its
// lower corner; clear_rows_kernel zeroes every row that is a corner of a
// marked cell (rows r with a mark at r - {0,1}^3): a warp walks one (z, y)
// line of rows 32 at a time and writes the dirty ones of each 32 as
// contiguous float4 runs.

__global__ void __launch_bounds__(256) mark_rows_kernel(const float* __restrict__ seg, long long cap,
                                                        const int64_t* __restrict__ n_dev, int nvx, int nvy, int nvz,
                                                        uint8_t* __restrict__ touched) {
  const long long n = segment_total(cap, n_dev);
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < n; s += stride) {
    const float* p = seg + 6 * s;
    const SegCorner c = segment_corners(__ldg(p), __ldg(p + 1), __ldg(p + 2), __ldg(p + 3), __ldg(p + 4),
                                        __ldg(p + 5), nvx, nvy, nvz);
    touched[((long long)c.z * nvy + c.y) * nvx + c.x] = 1;
  }
}

template <int F4>  // float4 per row; 0: runtime f4
__global__ void __launch_bounds__(256) clear_rows_kernel(float4* __restrict__ grid, int f4, int nvx, int nvy, int nvz,
                                                         const uint8_t* __restrict__ touched) {
  const int per_row = F4 ? F4 : f4;
  const int lines = nvy * nvz;  // rows of one (z, y) are contiguous in x
  const int lane = threadIdx.x & 31;
  const int warps = gridDim.x * (blockDim.x >> 5);
  // one warp per line; everything below is warp-uniform except x
  for (int line = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; line < lines; line += warps) {
    const int y = line % nvy, z = line / nvy;
    // the marks of the 4 lines (z - dz, y - dy) whose cells have this line's rows as corners
    const uint8_t* m00 = touched + (long long)line * nvx;
    const uint8_t* m01 = y > 0 ? m00 - nvx : nullptr;
    const uint8_t* m10 = z > 0 ? m00 - (long long)nvy * nvx : nullptr;
    const uint8_t* m11 = (y > 0 && z > 0) ? m10 - nvx : nullptr;
    float4* base = grid + (long long)line * nvx * per_row;
    unsigned carry = 0;  // the OR of the 4 marks at x - 1 for lane 0 (previous chunk's lane 31)
    for (int x0 = 0; x0 < nvx; x0 += 32) {
      const int x = x0 + lane;
      unsigned u = 0;
      if (x < nvx) {
        u = __ldg(m00 + x);
        if (m01) u |= __ldg(m01 + x);
        if (m10) u |= __ldg(m10 + x);
        if (m11) u |= __ldg(m11 + x);
      }
      const unsigned left = __shfl_up_sync(0xffffffffu, u, 1);
      const bool dirty = x < nvx && (u | (lane ? left : carry)) != 0;
      carry = __shfl_sync(0xffffffffu, u, 31);
      const unsigned m = __ballot_sync(0xffffffffu, dirty);
      if (m == 0) continue;
      float4* b = base + (long long)x0 * per_row;
      for (int e = lane; e < 32 * per_row; e += 32)
        if ((m >> (e / per_row)) & 1u) b[e] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
}

}  // namespace dv

using namespace dv;

extern "C" {

int dv_integrate_fwd(const float* voxels, int nvx, int nvy, int nvz, int channels, const float* coord_i,
                     const float* coord_o, long long coord_stride, long long n_seg, float* feature,
                     void* stream) {
  IntegrateArgs a{};
  a.grid = voxels;
  a.ci = coord_i;
  a.co = coord_o;
  a.stride = coord_stride;
  a.n_seg = n_seg;
  a.out = feature;
  a.nvx = nvx;
  a.nvy = nvy;
  a.nvz = nvz;
  a.C = channels;
  int st = check_common(a);
  if (st) return st;
  if (n_seg == 0) return DV_OK;
  DV_CHECK(voxels && feature && ((uintptr_t)voxels & 15) == 0 && ((uintptr_t)feature & 15) == 0, DV_ERR_ARG);
  const long long threads = n_seg * (channels / 4);
  integrate_fwd_kernel<<<ceil_div(threads, 256), 256, 0, (cudaStream_t)stream>>>(a);
  DV_TRY_LAUNCH();
  return DV_OK;
}

int dv_integrate_bwd(const float* grad_feature, int nvx, int nvy, int nvz, int channels, const float* coord_i,
                     const float* coord_o, long long coord_stride, long long n_seg, float* grad_voxels,
                     void* stream) {
  IntegrateArgs a{};
  a.grad_grid = grad_voxels;
  a.ci = coord_i;
  a.co = coord_o;
  a.stride = coord_stride;
  a.n_seg = n_seg;
  a.gin = grad_feature;
  a.nvx = nvx;
  a.nvy = nvy;
  a.nvz = nvz;
  a.C = channels;
  int st = check_common(a);
  if (st) return st;
  if (n_seg == 0) return DV_OK;
  DV_CHECK(grad_feature && grad_voxels && ((uintptr_t)grad_voxels & 15) == 0 && ((uintptr_t)grad_feature & 15) == 0,
           DV_ERR_ARG);
  const long long threads = n_seg * (channels / 4);
  integrate_bwd_kernel<<<ceil_div(threads, 256), 256, 0, (cudaStream_t)stream>>>(a);
  DV_TRY_LAUNCH();
  return DV_OK;
}

int dv_corner_rows(const float* coord_i, const float* coord_o, long long coord_stride, long long n_seg, int n_vert,
                   int64_t* rows, void* stream) {
  DV_CHECK(n_seg >= 0 && n_vert > 0 && coord_stride >= 3, DV_ERR_ARG);
  if (n_seg == 0) return DV_OK;
  DV_CHECK(coord_i && coord_o && rows, DV_ERR_ARG);
  corner_rows_kernel<<<ceil_div(n_seg, 256), 256, 0, (cudaStream_t)stream>>>(coord_i, coord_o, coord_stride, n_seg,
                                                                              n_vert, rows);
  DV_TRY_LAUNCH();
  return DV_OK;
}

int dv_integrate_table_fwd(const float* table, long long n_rows, int channels, const int64_t* rows,
                           const float* coord_i, const float* coord_o, long long coord_stride, long long n_seg,
                           float* feature, void* stream) {
  DV_CHECK(n_seg >= 0 && n_rows >= 0 && channels > 0 && (channels & 3) == 0 && coord_stride >= 3, DV_ERR_ARG);
  if (n_seg == 0) return DV_OK;
  DV_CHECK(table && rows && coord_i && coord_o && feature, DV_ERR_ARG);
  DV_CHECK(((uintptr_t)table & 15) == 0 && ((uintptr_t)feature & 15) == 0, DV_ERR_ARG);
  IntegrateArgs a{};
  a.grid = table;
  a.rows = rows;
  a.ci = coord_i;
  a.co = coord_o;
  a.stride = coord_stride;
  a.n_seg = n_seg;
  a.out = feature;
  a.C = channels;
  integrate_table_fwd_kernel<<<ceil_div(n_seg * (channels / 4), 256), 256, 0, (cudaStream_t)stream>>>(a);
  DV_TRY_LAUNCH();
  return DV_OK;
}

int dv_integrate_table_bwd(const float* grad_feature, long long n_rows, int channels, const int64_t* rows,
                           const float* coord_i, const float* coord_o, long long coord_stride, long long n_seg,
                           float* grad_table, void* stream) {
  DV_CHECK(n_seg >= 0 && n_rows >= 0 && channels > 0 && (channels & 3) == 0 && coord_stride >= 3, DV_ERR_ARG);
  if (n_seg == 0) return DV_OK;
  DV_CHECK(grad_feature && rows && coord_i && coord_o && grad_table, DV_ERR_ARG);
  DV_CHECK(((uintptr_t)grad_table & 15) == 0 && ((uintptr_t)grad_feature & 15) == 0, DV_ERR_ARG);
  IntegrateArgs a{};
  a.grad_grid = grad_table;
  a.rows = rows;
  a.ci = coord_i;
  a.co = coord_o;
  a.stride = coord_stride;
  a.n_seg = n_seg;
  a.gin = grad_feature;
  a.C = channels;
  integrate_table_bwd_kernel<<<ceil_div(n_seg * (channels / 4), 256), 256, 0, (cudaStream_t)stream>>>(a);
  DV_TRY_LAUNCH();
  return DV_OK;
}

int dv_mark_corner_rows(const float* seg, long long n_seg, const int64_t* n_seg_dev, int nvx, int nvy, int nvz,
                        uint8_t* touched, void* stream) {
  DV_CHECK(n_seg >= 0 && nvx > 0 && nvy > 0 && nvz > 0, DV_ERR_ARG);
  if (n_seg == 0) return DV_OK;
  DV_CHECK(seg && touched, DV_ERR_ARG);
  const unsigned need = ceil_div(n_seg, 256);
  const unsigned blocks = need < 152u * 8u ? need : 152u * 8u;
  mark_rows_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(seg, n_seg, n_seg_dev, nvx, nvy, nvz, touched);
  DV_TRY_LAUNCH();
  return DV_OK;
}

int dv_clear_marked_rows(float* grid, int channels, int nvx, int nvy, int nvz, uint8_t* touched, void* stream) {
  DV_CHECK(channels > 0 && (channels & 3) == 0 && nvx > 0 && nvy > 0 && nvz > 0, DV_ERR_ARG);
  DV_CHECK(grid && touched && ((uintptr_t)grid & 15) == 0, DV_ERR_ARG);
  DV_CHECK((long long)nvy * nvz < (1ll << 31), DV_ERR_ARG);
  const long long rows = (long long)nvx * nvy * nvz;
  // 1 block per SM: the clear runs beside the step's traversal on another
  // stream, and a grid that filled every SM's thread slots with grid-stride
  // blocks would keep the traversal's blocks from starting until it ended
  const unsigned need = ceil_div((long long)nvy * nvz, 8);  // 8 warps (lines) per block
  const unsigned blocks = need < 152u ? need : 152u;
  float4* g = reinterpret_cast<float4*>(grid);
  const cudaStream_t st = (cudaStream_t)stream;
  const int f4 = channels / 4;
  if (f4 == 8)
    clear_rows_kernel<8><<<blocks, 256, 0, st>>>(g, f4, nvx, nvy, nvz, touched);
  else if (f4 == 16)
    clear_rows_kernel<16><<<blocks, 256, 0, st>>>(g, f4, nvx, nvy, nvz, touched);
  else
    clear_rows_kernel<0><<<blocks, 256, 0, st>>>(g, f4, nvx, nvy, nvz, touched);
  DV_TRY_LAUNCH();
  if (cudaMemsetAsync(touched, 0, (size_t)rows, st) != cudaSuccess) return DV_ERR_CUDA;
  return DV_OK;
}

}  // extern "C"
