// Per-ray and compositing kernels of the training / offline path (plain FP32)
// and the C ABI of the segment-parallel decoder:
//   ray_pe         per-ray positional encoding and its contribution to mlp2's
//                  first layer (constant along a ray)
//   composite_fwd  per-ray alpha compositing (one warp per ray)
//   composite_bwd  per-segment dL/dsigma, dL/dcolor from dL/drgb
// Reference semantics: model/diver.py:183-207 (render), train.py:84-85,109-113
// (loss).  The decoder kernels themselves are in decode.cuh.
#include "decode.cuh"

namespace dv {

template <int W, int D1>
__global__ void __launch_bounds__(128) ray_pe_kernel(const DecodeArgs a) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= a.B) return;
  float pe[PE_PAD];
  pos_enc(__ldg(a.dirs + 3 * b), __ldg(a.dirs + 3 * b + 1), __ldg(a.dirs + 3 * b + 2), pe);
#pragma unroll
  for (int k = 0; k < PE_PAD; k += 4)
    *reinterpret_cast<float4*>(a.pe_feat + (long long)b * PE_PAD + k) = make_float4(pe[k], pe[k + 1], pe[k + 2], pe[k + 3]);
  const float* Wt = a.params + a.w_off[D1 + 1] + W * W;  // rows W .. W+26 of [W+27][W]
  const float* bias = a.params + a.b_off[D1 + 1];
  float* out = a.pe_out + (long long)b * W;
#pragma unroll 4
  for (int j = 0; j < W; ++j) {
    float acc = __ldg(bias + j);
    for (int k = 0; k < PE_DIM; ++k) acc = fmaf(pe[k], __ldg(Wt + k * W + j), acc);
    out[j] = acc;
  }
}

// ---- compositing -------------------------------------------------------------

__device__ __forceinline__ float warp_incl_scan(float v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const float y = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += y;
  }
  return v;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Kahan-compensated running sum.
struct Kahan {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float y = x - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
};

// rgb = sum_i w_i c_i (+ T_final for a white background), w_i = alpha_i T_i,
// alpha_i = 1 - exp(-relu(sigma_i)), T_i = exp(-sum_{j<i} relu(sigma_j)):
// the reference's render (model/diver.py:295-319) with the transmittance kept
// in log space (a compensated sum of relu(sigma), exact because
// log(1 - alpha) = -relu(sigma)) instead of a running product.
//
// OCC: instead of colours, the per-segment weight w_i goes into an occupancy
// map: alpha_map[cell] = max(alpha_map[cell], w_i) over the voxel cell
// min(int(p0 + 1e-4), int(p1 + 1e-4)) of each segment whose cell lies in
// [pad, N-1-pad]^3, flattened x + y N + z N^2 (prune.py:114-131, the
// reference's torch_scatter max).  w_i >= 0, so the float maximum is an
// integer atomicMax on the bit patterns of a map that starts at +0.
template <bool OCC>
__global__ void __launch_bounds__(256) composite_kernel(const DecodeArgs a) {
  const int ray = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (ray >= a.B) return;
  const long long beg = a.offsets[ray], end = a.offsets[ray + 1];
  Kahan logt;
  float r = 0.f, g = 0.f, bl = 0.f, reg = 0.f;
  for (long long base = beg; base < end; base += 32) {
    const long long i = base + lane;
    const bool valid = i < end;
    const float4 v = valid ? a.out4[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float s = fmaxf(v.x, 0.f);
    const float incl = warp_incl_scan(s);
    const float excl = incl - s;
    const float T = expf(-(logt.s + excl) + logt.c);
    const float w = -expm1f(-s) * T;
    if (OCC) {
      if (valid) {
        const float* p = a.seg + i * 6;
        const int n = a.occ_n, lo = a.occ_pad, hi = a.occ_n - 1 - a.occ_pad;
        const int cx = min((int)__fadd_rn(p[0], 1e-4f), (int)__fadd_rn(p[3], 1e-4f));
        const int cy = min((int)__fadd_rn(p[1], 1e-4f), (int)__fadd_rn(p[4], 1e-4f));
        const int cz = min((int)__fadd_rn(p[2], 1e-4f), (int)__fadd_rn(p[5], 1e-4f));
        if (cx >= lo && cx <= hi && cy >= lo && cy <= hi && cz >= lo && cz <= hi)
          atomicMax(reinterpret_cast<int*>(a.alpha_map) + ((long long)cz * n + cy) * n + cx, __float_as_int(w));
      }
      logt.add(__shfl_sync(0xffffffffu, incl, 31));
      continue;
    }
    r = fmaf(w, v.y, r);
    g = fmaf(w, v.z, g);
    bl = fmaf(w, v.w, bl);
    if (valid) reg += log1pf(v.x * v.x * 2.f);
    logt.add(__shfl_sync(0xffffffffu, incl, 31));
  }
  if (OCC) return;
  r = warp_sum(r);
  g = warp_sum(g);
  bl = warp_sum(bl);
  reg = warp_sum(reg);
  if (lane == 0) {
    const float tf = expf(-logt.s + logt.c);
    const float bg = a.white_back ? tf : 0.f;
    a.rgb[3 * ray] = r + bg;
    a.rgb[3 * ray + 1] = g + bg;
    a.rgb[3 * ray + 2] = bl + bg;
    if (a.t_final) a.t_final[ray] = tf;
    if (a.reg_sum) a.reg_sum[ray] = reg;
  }
}

// dL/ds_i = T_{i+1} (g . c_i) - g . rgb + sum_{j<=i} w_j (g . c_j), with s = relu(sigma);
// dL/dc_i = w_i g; plus the sparsity term l_s/(B M) * 2 sigma / (0.5 + sigma^2)
// (train.py:84-85: mean of log(1 + sigma^2/0.5) over the padded [B, M]).
__global__ void __launch_bounds__(256) composite_bwd_kernel(const DecodeArgs a, float4* d4) {
  const int ray = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (ray >= a.B) return;
  const long long beg = a.offsets[ray], end = a.offsets[ray + 1];
  const float g0 = a.g_rgb[3 * ray], g1 = a.g_rgb[3 * ray + 1], g2 = a.g_rgb[3 * ray + 2];
  const float grgb = g0 * a.rgb[3 * ray] + g1 * a.rgb[3 * ray + 1] + g2 * a.rgb[3 * ray + 2];
  const float rc = a.reg_scale ? a.reg_coef * *a.reg_scale : a.reg_coef;
  Kahan logt;
  float carry = 0.f;  // sum_{j < chunk} w_j (g . c_j)
  for (long long base = beg; base < end; base += 32) {
    const long long i = base + lane;
    const bool valid = i < end;
    const float4 v = valid ? a.out4[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float s = fmaxf(v.x, 0.f);
    const float incl = warp_incl_scan(s);
    const float excl = incl - s;
    const float T = expf(-(logt.s + excl) + logt.c);
    const float Tn = expf(-(logt.s + incl) + logt.c);
    const float w = -expm1f(-s) * T;
    const float gc = g0 * v.y + g1 * v.z + g2 * v.w;
    const float pincl = warp_incl_scan(w * gc) + carry;
    float ds = Tn * gc - grgb + pincl;
    float dsig = v.x > 0.f ? ds : 0.f;
    dsig += rc * 2.f * v.x / (0.5f + v.x * v.x);
    if (valid) d4[i] = make_float4(dsig, w * g0, w * g1, w * g2);
    logt.add(__shfl_sync(0xffffffffu, incl, 31));
    carry = __shfl_sync(0xffffffffu, pincl, 31);
  }
}

static int sm_count() {
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n > 0 ? n : 1;
}

// Sum over the 1024 threads of a block (tree through shared memory); every
// thread gets the total.
__device__ __forceinline__ float block_sum_1024(float v) {
  __shared__ float part[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) part[w] = v;
  __syncthreads();
  v = part[lane];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// The sparsity term's mean over the padded [B, M] (model/diver.py:199-205:
// the per-ray sums divided by B * M, M the longest ray, at least 1), M read on
// the device when m_dev is given; inv_m = 1 / M for the backward.  One block.
__global__ void __launch_bounds__(1024) reg_mean_kernel(const float* __restrict__ reg, int B, const int* m_dev,
                                                        float m_host, float* out, float* inv_m) {
  float v = 0.f;
  for (int i = threadIdx.x; i < B; i += 1024) v += reg[i];
  v = block_sum_1024(v);
  if (threadIdx.x == 0) {
    const float m = fmaxf(m_dev ? (float)*m_dev : m_host, 1.f);
    out[0] = v / ((float)B * m);
    inv_m[0] = 1.f / m;
  }
}

// Training loss of train.py:84-85,109-113: mean((x - y)^2) over n values plus
// l_s times the sparsity term (a device scalar, or none).  One block.
__global__ void __launch_bounds__(1024) l2_loss_fwd_kernel(const float* __restrict__ x, const float* __restrict__ y,
                                                           long long n, const float* reg, float l_s, float* loss) {
  float v = 0.f;
  for (long long i = threadIdx.x; i < n; i += 1024) {
    const float d = x[i] - y[i];
    v = fmaf(d, d, v);
  }
  v = block_sum_1024(v);
  if (threadIdx.x == 0) loss[0] = v / (float)n + (reg ? l_s * reg[0] : 0.f);
}

// Its gradients for the incoming dL (a device scalar): dx = 2 (x - y) / n * dL,
// dreg = l_s * dL.
__global__ void l2_loss_bwd_kernel(const float* __restrict__ x, const float* __restrict__ y, long long n,
                                   const float* g, float l_s, float* dx, float* dreg) {
  const float gg = g[0];
  const float c = 2.f * gg / (float)n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    dx[i] = c * (x[i] - y[i]);
  if (blockIdx.x == 0 && threadIdx.x == 0 && dreg) dreg[0] = l_s * gg;
}

}  // namespace dv

using namespace dv;

// Decoder kinds: 32 = DIVeR32 (width 32, two hidden layers), 64 = DIVeR64
// (width 64, one hidden layer); channels 32 or 64.
static int fill_layers(DecodeArgs& a, int kind, int channels) {
  int W, D1;
  if (kind == 32) {
    W = 32;
    D1 = 2;
  } else if (kind == 64) {
    W = 64;
    D1 = 1;
  } else {
    return DV_ERR_ARG;
  }
  if (channels != 32 && channels != 64) return DV_ERR_ARG;
  int dims[MAX_LAYERS][2];
  int n = 0;
  dims[n][0] = channels;
  dims[n++][1] = W;
  for (int d = 1; d < D1; ++d) {
    dims[n][0] = W;
    dims[n++][1] = W;
  }
  dims[n][0] = W;
  dims[n++][1] = W + 1;
  dims[n][0] = W + PE_DIM;
  dims[n++][1] = W;
  dims[n][0] = W;
  dims[n++][1] = 3;
  int off = 0;
  for (int l = 0; l < n; ++l) {
    a.w_off[l] = off;
    a.b_off[l] = off + dims[l][0] * pad4(dims[l][1]);
    off = a.b_off[l] + pad4(dims[l][1]);
  }
  a.n_params = off;
  return DV_OK;
}

extern "C" {

int dv_decoder_param_count(int kind, int channels) {
  DecodeArgs a{};
  if (fill_layers(a, kind, channels)) return -1;
  return a.n_params;
}

int dv_ray_pe(int kind, int channels, const float* params, int batch, const float* dirs, float* pe_feat, float* pe_out,
              void* stream) {
  DecodeArgs a{};
  DV_CHECK(fill_layers(a, kind, channels) == DV_OK && batch >= 0, DV_ERR_ARG);
  if (batch == 0) return DV_OK;
  DV_CHECK(params && dirs && pe_feat && pe_out, DV_ERR_ARG);
  a.params = params;
  a.B = batch;
  a.dirs = dirs;
  a.pe_feat = pe_feat;
  a.pe_out = pe_out;
  cudaStream_t st = (cudaStream_t)stream;
  if (kind == 32) ray_pe_kernel<32, 2><<<ceil_div(batch, 128), 128, 0, st>>>(a);
  else ray_pe_kernel<64, 1><<<ceil_div(batch, 128), 128, 0, st>>>(a);
  DV_TRY_LAUNCH();
  return DV_OK;
}

int dv_decode_fwd(int kind, int channels, const float* params, const float* voxels, int nvx, int nvy, int nvz,
                  const float* seg, const int* seg_ray, long long n_seg, const int64_t* n_seg_dev,
                  const float* pe_out, float* out4, void* stream) {
  DecodeArgs a{};
  DV_CHECK(fill_layers(a, kind, channels) == DV_OK && n_seg >= 0, DV_ERR_ARG);
  if (n_seg == 0) return DV_OK;
  DV_CHECK(params && voxels && seg && seg_ray && pe_out && out4, DV_ERR_ARG);
  DV_CHECK(((uintptr_t)voxels & 15) == 0 && ((uintptr_t)out4 & 15) == 0 && ((uintptr_t)params & 15) == 0, DV_ERR_ARG);
  a.grid = voxels;
  a.nvx = nvx;
  a.nvy = nvy;
  a.nvz = nvz;
  a.seg = seg;
  a.seg_ray = seg_ray;
  a.S = n_seg;
  a.S_dev = n_seg_dev;
  a.params = params;
  a.pe_out = const_cast<float*>(pe_out);
  a.out4 = reinterpret_cast<float4*>(out4);
  cudaStream_t st = (cudaStream_t)stream;
  const int sms = sm_count();
  if (kind == 32 && channels == 32) return decode_fwd_v32c32(a, st, sms);
  if (kind == 64 && channels == 32) return decode_fwd_v64c32(a, st, sms);
  if (kind == 64 && channels == 64) return decode_fwd_v64c64(a, st, sms);
  return DV_ERR_UNSUPPORTED;
}

int dv_composite_fwd(int batch, const int64_t* offsets, const float* out4, int white_back, float* rgb, float* t_final,
                     float* reg_sum, void* stream) {
  DV_CHECK(batch >= 0, DV_ERR_ARG);
  if (batch == 0) return DV_OK;
  DV_CHECK(offsets && out4 && rgb, DV_ERR_ARG);
  DecodeArgs a{};
  a.B = batch;
  a.offsets = offsets;
  a.out4 = reinterpret_cast<float4*>(const_cast<float*>(out4));
  a.white_back = white_back;
  a.rgb = rgb;
  a.t_final = t_final;
  a.reg_sum = reg_sum;
  composite_kernel<false><<<ceil_div((long long)batch * 32, 256), 256, 0, (cudaStream_t)stream>>>(a);
  DV_TRY_LAUNCH();
  return DV_OK;
}

int dv_occupancy_max(int batch, const int64_t* offsets, const float* out4, const float* seg, int voxel_num, int pad,
                     float* alpha_map, void* stream) {
  DV_CHECK(batch >= 0 && voxel_num > 0 && pad >= 0, DV_ERR_ARG);
  if (batch == 0) return DV_OK;
  DV_CHECK(offsets && out4 && seg && alpha_map, DV_ERR_ARG);
  DecodeArgs a{};
  a.B = batch;
  a.offsets = offsets;
  a.out4 = reinterpret_cast<float4*>(const_cast<float*>(out4));
  a.seg = seg;
  a.occ_n = voxel_num;
  a.occ_pad = pad;
  a.alpha_map = alpha_map;
  composite_kernel<true><<<ceil_div((long long)batch * 32, 256), 256, 0, (cudaStream_t)stream>>>(a);
  DV_TRY_LAUNCH();
  return DV_OK;
}

int dv_composite_bwd(int batch, const int64_t* offsets, const float* out4, const float* rgb, const float* grad_rgb,
                     float reg_coef, const float* reg_scale, float* d4, void* stream) {
  DV_CHECK(batch >= 0, DV_ERR_ARG);
  if (batch == 0) return DV_OK;
  DV_CHECK(offsets && out4 && rgb && grad_rgb && d4, DV_ERR_ARG);
  DecodeArgs a{};
  a.B = batch;
  a.offsets = offsets;
  a.out4 = reinterpret_cast<float4*>(const_cast<float*>(out4));
  a.rgb = const_cast<float*>(rgb);
  a.g_rgb = grad_rgb;
  a.reg_coef = reg_coef;
  a.reg_scale = reg_scale;
  composite_bwd_kernel<<<ceil_div((long long)batch * 32, 256), 256, 0, (cudaStream_t)stream>>>(
      a, reinterpret_cast<float4*>(d4));
  DV_TRY_LAUNCH();
  return DV_OK;
}

int dv_decode_bwd(int kind, int channels, const float* params, const float* voxels, int nvx, int nvy, int nvz,
                  const float* seg, const int* seg_ray, long long n_seg, const int64_t* n_seg_dev,
                  const float* pe_feat, const float* pe_out, const float* d4, float* grad_voxels, float* grad_params,
                  void* stream) {
  DecodeArgs a{};
  DV_CHECK(fill_layers(a, kind, channels) == DV_OK && n_seg >= 0, DV_ERR_ARG);
  if (n_seg == 0) return DV_OK;
  DV_CHECK(params && voxels && seg && seg_ray && pe_feat && pe_out && d4 && grad_voxels && grad_params, DV_ERR_ARG);
  DV_CHECK(((uintptr_t)voxels & 15) == 0 && ((uintptr_t)grad_voxels & 15) == 0 && ((uintptr_t)d4 & 15) == 0,
           DV_ERR_ARG);
  a.grid = voxels;
  a.nvx = nvx;
  a.nvy = nvy;
  a.nvz = nvz;
  a.seg = seg;
  a.seg_ray = seg_ray;
  a.S = n_seg;
  a.S_dev = n_seg_dev;
  a.params = params;
  a.pe_feat = const_cast<float*>(pe_feat);
  a.pe_out = const_cast<float*>(pe_out);
  a.d4 = reinterpret_cast<const float4*>(d4);
  a.grad_grid = grad_voxels;
  a.grad_params = grad_params;
  cudaStream_t st = (cudaStream_t)stream;
  const int sms = sm_count();
  if (kind == 32 && channels == 32) return decode_bwd_v32c32(a, st, sms);
  if (kind == 64 && channels == 32) return decode_bwd_v64c32(a, st, sms);
  if (kind == 64 && channels == 64) return decode_bwd_v64c64(a, st, sms);
  return DV_ERR_UNSUPPORTED;
}

int dv_reg_mean(int batch, const float* reg, const int* max_dev, float max_host, float* mean, float* inv_max,
                void* stream) {
  DV_CHECK(batch >= 0 && reg && mean && inv_max, DV_ERR_ARG);
  reg_mean_kernel<<<1, 1024, 0, (cudaStream_t)stream>>>(reg, batch, max_dev, max_host, mean, inv_max);
  DV_TRY_LAUNCH();
  return DV_OK;
}

int dv_l2_loss_fwd(long long n, const float* x, const float* y, const float* reg, float l_s, float* loss,
                   void* stream) {
  DV_CHECK(n > 0 && x && y && loss, DV_ERR_ARG);
  l2_loss_fwd_kernel<<<1, 1024, 0, (cudaStream_t)stream>>>(x, y, n, reg, l_s, loss);
  DV_TRY_LAUNCH();
  return DV_OK;
}

int dv_l2_loss_bwd(long long n, const float* x, const float* y, const float* grad, float l_s, float* dx, float* dreg,
                   void* stream) {
  DV_CHECK(n > 0 && x && y && grad && dx, DV_ERR_ARG);
  const long long blocks = std::min<long long>((n + 255) / 256, 4LL * 152);
  l2_loss_bwd_kernel<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(x, y, n, grad, l_s, dx, dreg);
  DV_TRY_LAUNCH();
  return DV_OK;
}

}  // extern "C"
