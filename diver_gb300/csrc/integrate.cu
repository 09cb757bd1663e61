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

static int check_common(const IntegrateArgs& a) {
  if (a.n_seg < 0 || a.C <= 0 || (a.C & 3) || a.nvx <= 0 || a.nvy <= 0 || a.nvz <= 0 || a.stride < 3) return DV_ERR_ARG;
  if (a.n_seg > 0 && (!a.ci || !a.co)) return DV_ERR_ARG;
  return DV_OK;
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

}  // extern "C"
