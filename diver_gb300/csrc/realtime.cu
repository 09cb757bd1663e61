// Real-time fused decoder: per pixel, up to 8 recorded hits per call, the
// closed-form integral of the sparse feature table, the folded MLP, and
// front-to-back compositing with the reference's skip (alpha < 1e-2) and
// early-termination (T < 1e-2) rules.
// Reference: utils/mlp_evaluation/src/mlp_eval.cu:32-231 (DIVeR32) and
// utils/mlp_evaluation64/src/mlp_eval.cu:32-231 (DIVeR64).
//
// Differences from the reference, by design: no process-global state (the
// reference binds a 3D texture and a __constant__ array in upload_weight);
// the voxel index map and the weights are per-model device buffers passed to
// every call, so several models can be resident.  The clamped texture lookup
// becomes an explicit clamp.  The weights are re-laid out once at upload
// (dv_realtime_pack) so every row is float4 aligned and they are staged in
// shared memory.  Math uses expf/sincosf, not the fast intrinsics.
#include "common.cuh"
#include "integrate.cuh"
#include "mlp.cuh"
#include "realtime.cuh"

namespace dv {

template <int W, int FIRST>
__global__ void pack_kernel(const float* __restrict__ ref, float* __restrict__ out) {
  using L = RtLayout<W, FIRST>;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= L::size) return;
  // reference offsets (convert.py:94-140)
  const int r0 = FIRST ? 32 : 0;      // weight0^T [33][W]: bias row then 32 rows
  const int r1 = r0 + 33 * W;         // weight1 [W+1]: sigma bias, weights
  const int r2 = r1 + W + 1;          // w2^T [1+W+27][W]
  const int r3 = r2 + (1 + W + 27) * W;  // weight3^T [W+1][3]
  float v = 0.f;
  int i = tid;
  if (FIRST && i < 32) {
    v = ref[i];
  } else if (i >= L::l0_b && i < L::l0_w) {
    v = ref[r0 + (i - L::l0_b)];
  } else if (i >= L::l0_w && i < L::sig) {
    v = ref[r0 + W + (i - L::l0_w)];
  } else if (i >= L::sig && i < L::sig + W) {
    v = ref[r1 + 1 + (i - L::sig)];
  } else if (i == L::sig + W) {
    v = ref[r1];
  } else if (i >= L::l2_b && i < L::l2_w) {
    v = ref[r2 + (i - L::l2_b)];
  } else if (i >= L::l2_w && i < L::l2_pe) {
    v = ref[r2 + W + (i - L::l2_w)];
  } else if (i >= L::l2_pe && i < L::l3_b) {
    const int k = (i - L::l2_pe) / W, j = (i - L::l2_pe) % W;
    v = k < PE_DIM ? ref[r2 + (1 + W + pe_ref_row(k)) * W + j] : 0.f;
  } else if (i >= L::l3_b && i < L::l3_b + 3) {
    v = ref[r3 + (i - L::l3_b)];
  } else if (i >= L::l3_w) {
    const int row = (i - L::l3_w) / 4, j = (i - L::l3_w) % 4;
    v = j < 3 ? ref[r3 + 3 * (1 + row) + j] : 0.f;
  }
  out[tid] = v;
}

struct RtArgs {
  int batch;
  const float* coords;   // [8][B][6]
  const float* feats;    // [F][32]
  const int* vmap;       // [(N+1)^3]
  int ms;                // N+1
  const float* params;   // aligned layout
  const float* v;        // [B][3]
  float* rgba;           // [B][4]
  uint8_t* finish;       // [B]
};

__device__ __forceinline__ int clampi(int x, int hi) { return x < 0 ? 0 : (x > hi ? hi : x); }

// One recorded hit (segment p0 -> p1 in fine voxel units) of one pixel:
// integral of the sparse feature table, the folded MLP, and front-to-back
// compositing into acc (rgb, T).  Returns false when the pixel is finished
// (T < 1e-2).  Shared by the per-round kernel and the fused frame kernel so
// both perform the same arithmetic.
template <int W, int FIRST>
__device__ __forceinline__ bool rt_eval_hit(const float* __restrict__ sw, float* X, float* H, const float* pe,
                                            const float* __restrict__ feats, const int* __restrict__ vmap, int ms,
                                            float x0, float y0, float z0, float x1, float y1, float z1,
                                            float4& acc) {
  using L = RtLayout<W, FIRST>;
  float y[W + 4];
  // corner weights; the index clamp of segment_corners is replaced by the
  // texture-style clamp of each lookup (mlp_eval.cu:112-118)
  const SegCorner sc = segment_corners(x0, y0, z0, x1, y1, z1, 1 << 30, 1 << 30, 1 << 30);
  float f[32];
#pragma unroll
  for (int k = 0; k < 32; ++k) f[k] = FIRST ? sw[L::b_in + k] : 0.f;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int x = clampi(sc.x + (j & 1), ms - 1);
    const int yy = clampi(sc.y + ((j >> 1) & 1), ms - 1);
    const int z = clampi(sc.z + (j >> 2), ms - 1);
    const int idx = __ldg(vmap + ((long long)z * ms + yy) * ms + x);
    const float4* row = reinterpret_cast<const float4*>(feats + (long long)idx * 32);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const float4 v = __ldg(row + q);
      f[4 * q] = fmaf(sc.w[j], v.x, f[4 * q]);
      f[4 * q + 1] = fmaf(sc.w[j], v.y, f[4 * q + 1]);
      f[4 * q + 2] = fmaf(sc.w[j], v.z, f[4 * q + 2]);
      f[4 * q + 3] = fmaf(sc.w[j], v.w, f[4 * q + 3]);
    }
  }
#pragma unroll
  for (int k = 0; k < 32; ++k) X[k] = FIRST ? fmaxf(f[k], 0.f) : f[k];
  dense_fwd_s<W, false>(sw + L::l0_w, sw + L::l0_b, X, 32, y);
#pragma unroll
  for (int k = 0; k < W; ++k) H[k] = fmaxf(y[k], 0.f);
  float sigma = sw[L::sig + W];
#pragma unroll 8
  for (int k = 0; k < W; ++k) sigma = fmaf(sw[L::sig + k], H[k], sigma);
  const float alpha = 1.f - expf(-fmaxf(sigma, 0.f));
  if (alpha < 1e-2f) return true;
  dense_fwd_s<W, false>(sw + L::l2_w, sw + L::l2_b, H, W, y);
#pragma unroll
  for (int k = 0; k < PE_DIM; ++k) {
    const float p = pe[k];
#pragma unroll
    for (int j = 0; j < W; j += 4) {
      const float4 w = *reinterpret_cast<const float4*>(sw + L::l2_pe + k * W + j);
      y[j] = fmaf(p, w.x, y[j]);
      y[j + 1] = fmaf(p, w.y, y[j + 1]);
      y[j + 2] = fmaf(p, w.z, y[j + 2]);
      y[j + 3] = fmaf(p, w.w, y[j + 3]);
    }
  }
#pragma unroll
  for (int k = 0; k < W; ++k) X[k] = fmaxf(y[k], 0.f);
  float o[4];
  dense_fwd_s<4, false>(sw + L::l3_w, sw + L::l3_b, X, W, o);
  const float wgt = acc.w * alpha;
  acc.x += wgt * sigmoidf_acc(o[0]);
  acc.y += wgt * sigmoidf_acc(o[1]);
  acc.z += wgt * sigmoidf_acc(o[2]);
  acc.w = acc.w * (1.f - alpha);
  return !(acc.w < 1e-2f);
}

template <int W, int FIRST>
__device__ __forceinline__ void stage_weights(const float* __restrict__ params, float* sw) {
  using L = RtLayout<W, FIRST>;
  for (int i = threadIdx.x; i < L::size / 4; i += blockDim.x)
    reinterpret_cast<float4*>(sw)[i] = __ldg(reinterpret_cast<const float4*>(params) + i);
  __syncthreads();
}

template <int W, int FIRST>
__global__ void __launch_bounds__(128) mlp_eval_kernel(const RtArgs a) {
  using L = RtLayout<W, FIRST>;
  extern __shared__ __align__(16) float smem[];
  float* sw = smem;
  float* rows = smem + L::size;
  stage_weights<W, FIRST>(a.params, sw);
  // one row per thread serves as the input of every layer: each layer's output
  // is in registers before the row is rewritten (integrated feature, h1, h2)
  float* X = rows + threadIdx.x * (W + 4);
  float* H = X;
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= a.batch || a.finish[b]) return;
  float pe[PE_PAD];
  pos_enc(__ldg(a.v + 3 * b), __ldg(a.v + 3 * b + 1), __ldg(a.v + 3 * b + 2), pe);
  float4 acc = reinterpret_cast<float4*>(a.rgba)[b];
  const long long stride = (long long)a.batch * 6;
  for (int hit = 0; hit < 8; ++hit) {
    const float* c = a.coords + hit * stride + (long long)b * 6;
    if (c[0] < 0.f) {
      a.finish[b] = 1;
      break;
    }
    if (!rt_eval_hit<W, FIRST>(sw, X, H, pe, a.feats, a.vmap, a.ms, c[0], c[1], c[2], c[3], c[4], c[5], acc)) {
      a.finish[b] = 1;
      break;
    }
  }
  reinterpret_cast<float4*>(a.rgba)[b] = acc;
}

// Whole frame in one launch: per pixel, the octree first hit, then rounds of
// (walk the fine occupancy mask to the next 8 occupied voxels, decode them)
// until the ray leaves the grid or T < 1e-2.  The per-ray arithmetic and its
// order are those of the host loop aabb_intersect + rounds of (ray_march,
// mlp_eval) (eval_rt.py:115-122); the rounds simply continue inside the
// kernel, with the hits in shared memory instead of a coords buffer and no
// host round trip between them.
struct RtFrameArgs {
  int batch;
  const float* v;        // [B][3] unit directions
  const float* center;   // [3] camera centre, fine voxel units (device)
  const uint8_t* oct;    // octree levels (scales 64, 16, 4), coarsest first
  long long oct_cells;
  const uint8_t* mask;   // [N][N][N] fine occupancy
  int N;
  const float* feats;
  const int* vmap;
  int ms;
  const float* params;
  float* rgba;           // [B][4] (rgb, T)
};

template <int W, int FIRST, bool FAST>
__device__ __forceinline__ void rt_frame_ray(const RtFrameArgs& a, const float* sw, float* X, float* H,
                                             float* hit_slots, int b, float3 p, const float3 d, float4& acc) {
  const float3 s = make_float3(step_sign(d.x), step_sign(d.y), step_sign(d.z));
  const float3 r = FAST ? make_float3(__frcp_rn(d.x), __frcp_rn(d.y), __frcp_rn(d.z)) : d;
  // octree: level 0 cells of 64^3 voxels, descend x4 on an occupied cell
  int m = a.N / 64;
  long long off = 0;
  float3 last = p;
  const int ocap = walk_cap((float)a.N, 0.f, 0.f) + 6;  // all octree levels (see octree_descend)
  int steps = 0;
  while (m < a.N) {
    if (steps++ == ocap) {
      note_cap_hit();
      return;
    }
    last = p;
    float3 q;
    float dt;
    grid_step<FAST>(last, d, r, s, q, dt);
    if (outside_closed(q, (float)m)) return;
    if (occupied(a.oct, off + cell_index1(last, q, m), a.oct_cells)) {
      off += (long long)m * m * m;
      last = make_float3(__fmul_rn(last.x, 4.f), __fmul_rn(last.y, 4.f), __fmul_rn(last.z, 4.f));
      p = last;
      m *= 4;
    } else {
      p = q;
    }
  }
  float pe[PE_PAD];
  pos_enc(d.x, d.y, d.z, pe);
  const float n = (float)a.N;
  const long long cells = (long long)a.N * a.N * a.N;
  // Rounds as in the host loop: march to the next 8 occupied voxels (kept in
  // this thread's shared-memory slots), then decode them.  Keeping the walk
  // and the decode in separate phases keeps a warp's lanes in the same phase;
  // decoding each hit as it is found would make every DDA step wait for the
  // lanes that decode.
  float* hits = hit_slots;  // [8][6] per thread
  const int cap = walk_cap(n, n, n);  // the fine walk over all rounds
  steps = 0;
  while (true) {
    int nh = 0;
    bool out = false;
    while (nh < 8) {
      if (steps++ == cap) {
        note_cap_hit();
        out = true;
        break;
      }
      float3 q;
      float dt;
      grid_step<FAST>(last, d, r, s, q, dt);
      if (outside_open(q, n)) {
        out = true;
        break;
      }
      if (occupied(a.mask, cell_index1(last, q, a.N), cells)) {
        float* h = hits + nh * 6;
        h[0] = last.x;
        h[1] = last.y;
        h[2] = last.z;
        h[3] = q.x;
        h[4] = q.y;
        h[5] = q.z;
        ++nh;
      }
      last = q;
    }
    for (int k = 0; k < nh; ++k) {
      const float* h = hits + k * 6;
      if (!rt_eval_hit<W, FIRST>(sw, X, H, pe, a.feats, a.vmap, a.ms, h[0], h[1], h[2], h[3], h[4], h[5], acc))
        return;
    }
    if (out) return;
  }
}

template <int W, int FIRST>
__global__ void __launch_bounds__(128) rt_frame_kernel(const RtFrameArgs a) {
  using L = RtLayout<W, FIRST>;
  extern __shared__ __align__(16) float smem[];
  float* sw = smem;
  float* rows = smem + L::size;
  stage_weights<W, FIRST>(a.params, sw);
  float* X = rows + threadIdx.x * (W + 4);  // one row for every layer's input (see mlp_eval_kernel)
  float* H = X;
  float* hit_slots = rows + blockDim.x * (W + 4) + threadIdx.x * 48;
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= a.batch) return;
  float4 acc = make_float4(0.f, 0.f, 0.f, 1.f);
  const float3 d = make_float3(__ldg(a.v + 3 * b), __ldg(a.v + 3 * b + 1), __ldg(a.v + 3 * b + 2));
  float3 p = make_float3(__ldg(a.center), __ldg(a.center + 1), __ldg(a.center + 2));
  float t;
  if (dir_ok(d) && box_entry(p, d, (float)a.N, t)) {
    p = make_float3(__fmul_rn(p.x, 0.015625f), __fmul_rn(p.y, 0.015625f), __fmul_rn(p.z, 0.015625f));
    if (a.N < (1 << 22) && recip_ok(d))
      rt_frame_ray<W, FIRST, true>(a, sw, X, H, hit_slots, b, p, d, acc);
    else
      rt_frame_ray<W, FIRST, false>(a, sw, X, H, hit_slots, b, p, d, acc);
  }
  reinterpret_cast<float4*>(a.rgba)[b] = acc;
}

template <int W, int FIRST>
int launch_mlp_eval(const RtArgs& a, cudaStream_t st) {
  using L = RtLayout<W, FIRST>;
  const size_t smem = (size_t)(L::size + 128 * (W + 4)) * sizeof(float);
  auto k = mlp_eval_kernel<W, FIRST>;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return DV_ERR_CUDA;
  k<<<ceil_div(a.batch, 128), 128, smem, st>>>(a);
  DV_TRY_LAUNCH();
  return DV_OK;
}

template <int W, int FIRST>
int launch_rt_frame(const RtFrameArgs& a, cudaStream_t st) {
  using L = RtLayout<W, FIRST>;
  const size_t smem = (size_t)(L::size + 128 * (W + 4) + 128 * 48) * sizeof(float);
  auto k = rt_frame_kernel<W, FIRST>;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return DV_ERR_CUDA;
  k<<<ceil_div(a.batch, 128), 128, smem, st>>>(a);
  DV_TRY_LAUNCH();
  return DV_OK;
}

}  // namespace dv

using namespace dv;

// Walks of this file's kernels that stopped at their step bound (summed by
// dv_walk_cap_hits in traverse.cu).
long long realtime_walk_cap_hits(int reset) {
  unsigned long long v = 0, w = 0;
  if (cudaMemcpyFromSymbol(&v, g_walk_cap_hits, sizeof(v)) != cudaSuccess) return -1;
  if (reset && cudaMemcpyToSymbol(g_walk_cap_hits, &w, sizeof(w)) != cudaSuccess) return -1;
  return (long long)v;
}

extern "C" {

int dv_realtime_packed_size(int width) {
  if (width == 32) return RtLayout<32, 1>::size;
  if (width == 64) return RtLayout<64, 0>::size;
  return -1;
}

int dv_realtime_pack(int width, const float* ref_params, float* packed, void* stream) {
  DV_CHECK((width == 32 || width == 64) && ref_params && packed, DV_ERR_ARG);
  DV_CHECK(((uintptr_t)packed & 15) == 0, DV_ERR_ARG);
  const int n = dv_realtime_packed_size(width);
  cudaStream_t st = (cudaStream_t)stream;
  if (width == 32) pack_kernel<32, 1><<<ceil_div(n, 256), 256, 0, st>>>(ref_params, packed);
  else pack_kernel<64, 0><<<ceil_div(n, 256), 256, 0, st>>>(ref_params, packed);
  DV_TRY_LAUNCH();
  return DV_OK;
}

int dv_mlp_eval(int width, int batch_size, const float* coords, const float* voxels, const int* voxel_map,
                int map_size, const float* packed_params, const float* v, float* rgba, uint8_t* finish,
                void* stream) {
  DV_CHECK((width == 32 || width == 64) && batch_size >= 0 && map_size > 0, DV_ERR_ARG);
  if (batch_size == 0) return DV_OK;
  DV_CHECK(coords && voxels && voxel_map && packed_params && v && rgba && finish, DV_ERR_ARG);
  DV_CHECK(((uintptr_t)voxels & 15) == 0 && ((uintptr_t)rgba & 15) == 0 && ((uintptr_t)packed_params & 15) == 0,
           DV_ERR_ARG);
  RtArgs a{batch_size, coords, voxels, voxel_map, map_size, packed_params, v, rgba, finish};
  cudaStream_t st = (cudaStream_t)stream;
  return width == 32 ? launch_mlp_eval<32, 1>(a, st) : launch_mlp_eval<64, 0>(a, st);
}

int dv_realtime_frame(int width, int batch_size, const float* v, const float* center, const uint8_t* octrees, int N,
                      const uint8_t* voxel_mask, const float* voxels, const int* voxel_map, int map_size,
                      const float* packed_params, float* rgba, void* stream) {
  DV_CHECK((width == 32 || width == 64) && batch_size >= 0 && N > 0 && N % 64 == 0 && map_size == N + 1, DV_ERR_ARG);
  if (batch_size == 0) return DV_OK;
  DV_CHECK(v && center && octrees && voxel_mask && voxels && voxel_map && packed_params && rgba, DV_ERR_ARG);
  DV_CHECK(((uintptr_t)voxels & 15) == 0 && ((uintptr_t)rgba & 15) == 0 && ((uintptr_t)packed_params & 15) == 0,
           DV_ERR_ARG);
  const long long n64 = N / 64, n16 = N / 16, n4 = N / 4;
  RtFrameArgs a{batch_size, v, center, octrees, n64 * n64 * n64 + n16 * n16 * n16 + n4 * n4 * n4, voxel_mask, N,
                voxels, voxel_map, map_size, packed_params, rgba};
  cudaStream_t st = (cudaStream_t)stream;
  return width == 32 ? launch_rt_frame<32, 1>(a, st) : launch_rt_frame<64, 0>(a, st);
}

}  // extern "C"
