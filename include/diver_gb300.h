/*
 * diver_gb300 — C ABI of the GB300 (sm_103a) DIVeR rendering hot path.
 *
 * Every entry point takes plain device pointers, sizes and scalars, plus the
 * CUDA stream to launch on (passed as void*, NULL = legacy default stream),
 * and returns a dv_status.  No entry point synchronises the device, exits the
 * process, or allocates memory unless its comment says so; output buffers are
 * owned by the caller.  All launches are stream-ordered.
 *
 * Coordinates are in voxel units (a point p in world space maps to
 * (p - xyzmin) / voxel_size).  Grids are stored [z][y][x][channel] with x
 * fastest, exactly as the reference's `voxels` parameter (model/diver.py:37).
 *
 * Reference citations are to files of the DIVeR project (lwwu2/diver).
 */
#ifndef DIVER_GB300_H
#define DIVER_GB300_H

#include <stdint.h>

#if defined(__GNUC__)
#define DV_API __attribute__((visibility("default")))
#else
#define DV_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum dv_status {
  DV_OK = 0,
  DV_ERR_ARG = 1,       /* bad size, NULL pointer or unsupported option */
  DV_ERR_CUDA = 2,      /* a CUDA call or launch failed */
  DV_ERR_OOM = 3,       /* an allocation (only in entry points that allocate) failed */
  DV_ERR_TIMEOUT = 4,   /* a bounded device wait ran out; see dv_last_device_error */
  DV_ERR_OVERFLOW = 5,  /* a capacity given by the caller was too small */
  DV_ERR_UNSUPPORTED = 6 /* the device is not sm_103 / feature not compiled */
} dv_status;

/* Library version (major*10000 + minor*100 + patch). */
DV_API int dv_version(void);

/* Name of a status code (static string). */
DV_API const char* dv_status_string(int status);

/* ------------------------------------------------------------------------
 * Ray–voxel traversal, training/offline path.
 * ------------------------------------------------------------------------ */

/*
 * Dense 3D-DDA: records the entry point of each ray into [0,N]^3 and every
 * grid-plane crossing after it.
 * Replaces ray_voxel_intersect_wrapper
 *   (utils/ray_voxel_intersection/src/ray_voxel_intersect.cu:154-172)
 * and the kernel it launches (same file :29-151).
 *   o, v          [batch][3] ray origins (world) and unit directions
 *   intersection  [batch][max_n][3]; the caller fills it with 0
 *   intersect_num [batch]; written (not accumulated)
 *   tns           [batch][max_n]; the caller fills it with -1
 *   max_count     optional device int (NULL to skip) that receives
 *                 max(intersect_num) through atomicMax; the caller zeroes it
 * Points beyond max_n are counted but not stored (the reference writes past
 * its buffer in that case).  As in the reference, a missed ray still gets its
 * clamped slab point in row 0 with count 0 and tns -1.
 */
DV_API int dv_ray_voxel_intersect(int batch_size, int max_n, float xyzmin, float xyzmax,
                           float voxel_num, float voxel_size, const float* o, const float* v,
                           float* intersection, int* intersect_num, float* tns, int* max_count,
                           void* stream);

/* Count-only pass of dv_ray_voxel_intersect (same walk, nothing stored but
 * intersect_num and max_count). */
DV_API int dv_ray_voxel_count(int batch_size, float xyzmin, float voxel_num, float voxel_size,
                       const float* o, const float* v, int* intersect_num, int* max_count,
                       void* stream);

/*
 * Masked 3D-DDA: records (entry, exit) of every voxel whose occupancy byte is
 * set, with the exit distance in tns.
 * Replaces masked_intersect_wrapper
 *   (utils/ray_voxel_intersection/src/ray_voxel_intersect.cu:323-341)
 * and masked_intersect_kernel (same file :192-319).
 *   mask          [M][M][M] bytes, M = int(voxel_num * mask_scale)
 *   intersection  [batch][max_n][6]; caller fills with 0
 *   tns           [batch][max_n]; caller fills with -1
 */
DV_API int dv_masked_intersect(int batch_size, int max_n, float xyzmin, float xyzmax, float voxel_num,
                        float voxel_size, float mask_scale, const float* o, const float* v,
                        const uint8_t* mask, float* intersection, int* intersect_num, float* tns,
                        int* max_count, void* stream);

/* Count-only pass of dv_masked_intersect. */
/* last_step (optional, int [batch]): the walk step (1-based) at which each ray
 * meets its last occupied voxel, 0 if none.  Given to the segment writers as
 * stop_step (optional), it lets their walk end there instead of at the far
 * side of the grid (same segments; nothing occupied lies beyond). */
DV_API int dv_masked_count(int batch_size, float xyzmin, float voxel_num, float voxel_size,
                    float mask_scale, const float* o, const float* v, const uint8_t* mask,
                    int* intersect_num, int* max_count, int* last_step, void* stream);

/*
 * Compacted (CSR) segment lists, the form DIVeR.extract_features builds with
 * boolean indexing (model/diver.py:86-103).  offsets[batch+1] is the exclusive
 * scan of the per-ray segment counts.  For every ray b, its segments are
 * written to rows offsets[b] .. offsets[b+1]-1 of
 *   seg      [S][6]  (entry xyz, exit xyz) in voxel units
 *   seg_t    [S]     distance (world units) or NULL
 *   seg_ray  [S]     ray index or NULL
 * Masked: one segment per occupied voxel, seg_t = exit distance (the masked
 *   kernel's tns).  Counts come from dv_masked_count.
 * Dense: consecutive crossing points pair into segments; ray b has
 *   max(count-1, 0) segments and seg_t is the entry distance (model/diver.py:
 *   95-103).  Counts come from dv_ray_voxel_count (minus one per ray).
 */
DV_API int dv_masked_segments(int batch_size, float xyzmin, float voxel_num, float voxel_size,
                       float mask_scale, const float* o, const float* v, const uint8_t* mask,
                       const int64_t* offsets, float* seg, float* seg_t, int* seg_ray,
                       const int* stop_step, void* stream);
DV_API int dv_dense_segments(int batch_size, float xyzmin, float voxel_num, float voxel_size,
                      const float* o, const float* v, const int64_t* offsets, float* seg,
                      float* seg_t, int* seg_ray, void* stream);

/*
 * Masked walk over a grid with per-axis extents (no counterpart in the
 * reference, whose grids are cubic: voxel_num is a scalar, model/diver.py:
 * 20-30).  xyzmin[3] (HOST array) is the world position of voxel corner
 * (0,0,0), dims[3] (HOST array) = (nx, ny, nz) voxels, mask [nz][ny][nx]
 * bytes.  With equal values on the three axes the arithmetic is exactly that
 * of dv_masked_count / dv_masked_segments (mask_scale 1).
 */
/* One walk instead of count + segments, for callers with fixed-capacity
 * buffers: ray b writes its segments (seg, t as dv_masked_segments) into rows
 * b * slot ... of seg_slots [batch * slot][6] / t_slots and its count into
 * intersect_num (max into max_count, optional); slot >= 3 * voxel_num + 3
 * (no ray crosses more grid planes).  Then dv_exclusive_scan of the counts and
 * dv_compact_slots give the CSR lists (seg, seg_t, seg_ray). */
DV_API int dv_masked_segments_slots(int batch_size, float xyzmin, float voxel_num, float voxel_size,
                                    float mask_scale, const float* o, const float* v, const uint8_t* mask,
                                    long long slot, float* seg_slots, float* t_slots, int* intersect_num,
                                    int* max_count, void* stream);
DV_API int dv_compact_slots(int batch_size, long long slot, const int64_t* offsets, const float* seg_slots,
                            const float* t_slots, float* seg, float* seg_t, int* seg_ray, void* stream);

DV_API int dv_masked_count_grid(int batch_size, const float* xyzmin, const int* dims, float voxel_size,
                                const float* o, const float* v, const uint8_t* mask, int* intersect_num,
                                int* max_count, int* last_step, void* stream);
DV_API int dv_masked_segments_grid(int batch_size, const float* xyzmin, const int* dims, float voxel_size,
                                   const float* o, const float* v, const uint8_t* mask,
                                   const int64_t* offsets, float* seg, float* seg_t, int* seg_ray,
                                   const int* stop_step, void* stream);

/* Per-ray segment counts for the dense pairing: max(intersect_num - 1, 0). */
DV_API int dv_dense_pair_counts(int batch_size, const int* intersect_num, int* seg_count, void* stream);

/*
 * Exclusive prefix sum of n int32 counts into n+1 int64 offsets
 * (offsets[n] = total).  scratch must hold dv_scan_scratch_bytes(n) bytes.
 */
/* Walks that stopped at their step bound since the last reset (no
 * counterpart in the reference, whose walks have no bound).  Every walk
 * (dense, masked, octree first hit, 8-hit march, the real-time frame) stops
 * after nx + ny + nz + 3 grid-plane steps, which no ray with a finite, nonzero
 * direction reaches (each step crosses one plane); rays with a non-finite or
 * zero direction are misses.  A nonzero count means some arithmetic case
 * broke that bound and its walk was cut short.  Synchronous (reads device
 * counters of the current device); reset = 1 zeroes them; -1 on a CUDA error. */
DV_API long long dv_walk_cap_hits(int reset);

DV_API long long dv_scan_scratch_bytes(long long n);
DV_API int dv_exclusive_scan(const int* counts, long long n, int64_t* offsets, void* scratch,
                      void* stream);

/* ------------------------------------------------------------------------
 * Feature integration.
 * ------------------------------------------------------------------------ */

/*
 * Mean of the trilinear interpolant of the 8 corner vectors over each
 * segment (closed form).  Replaces the reference's torch `integrate`
 * (utils/integrator.py:62-112).
 *   voxels    [nvz][nvy][nvx][channels] corner features, 16-byte aligned,
 *             channels a multiple of 4
 *   coord_i/o entry / exit points, 3 floats per row, rows coord_stride floats
 *             apart (3 for separate [S,3] arrays, 6 for the halves of [S,6])
 *   feature   [n_seg][channels] output
 * The lower corner is min(int(p_in + 1e-4), int(p_out + 1e-4)) per axis and
 * the upper corner is clamped to the last vertex, as in the reference.
 */
DV_API int dv_integrate_fwd(const float* voxels, int nvx, int nvy, int nvz, int channels,
                            const float* coord_i, const float* coord_o, long long coord_stride,
                            long long n_seg, float* feature, void* stream);

/*
 * Gradient of dv_integrate_fwd with respect to the corner features:
 * grad_voxels[corner] += w_corner * grad_feature, accumulated with atomics
 * (the caller zeroes grad_voxels).  This is the scatter the reference's
 * autograd performs through its 8 gathers (utils/integrator.py:80-85).
 */
DV_API int dv_integrate_bwd(const float* grad_feature, int nvx, int nvy, int nvz, int channels,
                            const float* coord_i, const float* coord_o, long long coord_stride,
                            long long n_seg, float* grad_voxels, void* stream);

/* Implicit stage (utils/integrator.py:3-59: integrate_mlp).  dv_corner_rows:
 * rows [n_seg][8] int64, the linear index (z * n_vert + y) * n_vert + x of
 * each segment's corner j (bit 0 = +x, bit 1 = +y, bit 2 = +z; lower corner
 * min(int(p0 + 1e-4), int(p1 + 1e-4)), upper corner clamped to n_vert - 1).
 * dv_integrate_table_fwd / _bwd: the integral of dv_integrate_fwd with corner
 * j read from row rows[s][j] of a feature table [n_rows][channels] (the
 * implicit MLP evaluated at the unique corners) instead of the grid; the
 * backward accumulates into grad_table. */
DV_API int dv_corner_rows(const float* coord_i, const float* coord_o, long long coord_stride,
                          long long n_seg, int n_vert, int64_t* rows, void* stream);
DV_API int dv_integrate_table_fwd(const float* table, long long n_rows, int channels,
                                  const int64_t* rows, const float* coord_i, const float* coord_o,
                                  long long coord_stride, long long n_seg, float* feature, void* stream);
DV_API int dv_integrate_table_bwd(const float* grad_feature, long long n_rows, int channels,
                                  const int64_t* rows, const float* coord_i, const float* coord_o,
                                  long long coord_stride, long long n_seg, float* grad_table,
                                  void* stream);

/* ------------------------------------------------------------------------
 * Decoder + compositing, training/offline path (plain FP32).
 *
 * kind 32 = DIVeR32 (mlp_point [32,2,33], mlp_view [32,1]),
 * kind 64 = DIVeR64 (mlp_point [64,1,65], mlp_view [64,1]); channels 32|64.
 * params: the packed torch form, every nn.Linear of mlp1 then mlp2 as
 * W^T [in][out4] (out4 = out rounded up to 4, extra columns 0) followed by the
 * bias [out4]; dv_decoder_param_count gives its length in floats.
 * Segments are the CSR lists of dv_masked_segments / dv_dense_segments.
 * n_seg_dev (optional, device int64, e.g. offsets + batch): the decode
 * kernels then read the segment count there, clamped to n_seg, which becomes
 * the capacity of the segment buffers; no host read of the count is needed,
 * so the launches can be recorded in a CUDA graph.
 * Replaces DIVeR.forward/decode/render (model/diver.py:159-207) and the
 * training loss (train.py:84-85,109-113).
 * ------------------------------------------------------------------------ */

DV_API int dv_decoder_param_count(int kind, int channels);

/* Per-ray positional encoding pe_feat [batch][28] (27 used) and its
 * contribution to mlp2's first layer incl. bias, pe_out [batch][width]. */
DV_API int dv_ray_pe(int kind, int channels, const float* params, int batch, const float* dirs,
                     float* pe_feat, float* pe_out, void* stream);

/* out4 [n_seg][4] = (sigma_raw, sigmoid rgb) per segment. */
DV_API int dv_decode_fwd(int kind, int channels, const float* params, const float* voxels, int nvx,
                         int nvy, int nvz, const float* seg, const int* seg_ray, long long n_seg,
                         const int64_t* n_seg_dev, const float* pe_out, float* out4, void* stream);

/* rgb [batch][3] (+ T_final if white_back), optional t_final [batch] and
 * reg_sum [batch] = sum over the ray's segments of log(1 + sigma^2 / 0.5). */
DV_API int dv_composite_fwd(int batch, const int64_t* offsets, const float* out4, int white_back,
                            float* rgb, float* t_final, float* reg_sum, void* stream);

/* Occupancy extraction (prune.py:86-131): with the rendering weights
 * w_i = alpha_i T_i of each ray's segments (out4 as from the decoder),
 * alpha_map [N][N][N] (x fastest, caller-initialised, e.g. zeros) becomes
 * max(alpha_map, w_i) at each segment's voxel min(int(p0 + 1e-4),
 * int(p1 + 1e-4)) that lies in [pad, N-1-pad]^3 — the reference's
 * torch_scatter max; voxel_mask = alpha_map > thresh is the pruned grid. */
DV_API int dv_occupancy_max(int batch, const int64_t* offsets, const float* out4, const float* seg,
                            int voxel_num, int pad, float* alpha_map, void* stream);

/* d4 [n_seg][4] = (dL/dsigma_raw, dL/drgb_seg) from grad_rgb [batch][3];
 * reg_coef multiplies d/dsigma log(1 + sigma^2/0.5), and so does *reg_scale
 * (device float, optional: a factor known only on the device, e.g.
 * dL/dreg / max segments per ray inside a captured CUDA graph). */
DV_API int dv_composite_bwd(int batch, const int64_t* offsets, const float* out4, const float* rgb,
                            const float* grad_rgb, float reg_coef, const float* reg_scale, float* d4,
                            void* stream);

/* The sparsity term's mean (model/diver.py:199-205): mean[0] = sum(reg[0..batch))
 * / (batch * M), M = max(*max_dev, 1) when max_dev is given (the longest ray,
 * kept on the device), else max(max_host, 1); inv_max[0] = 1 / M for the
 * backward's dv_composite_bwd reg_scale.  One launch, no host read. */
DV_API int dv_reg_mean(int batch, const float* reg, const int* max_dev, float max_host, float* mean,
                       float* inv_max, void* stream);

/* The training loss of train.py:84-85,109-113 and its gradients, as one launch
 * each (no counterpart in the reference, which composes them from torch ops):
 * loss[0] = mean over n of (x - y)^2 + l_s * reg[0] (reg optional);
 * dx = 2 (x - y) / n * grad[0], dreg[0] = l_s * grad[0] (dreg optional). */
DV_API int dv_l2_loss_fwd(long long n, const float* x, const float* y, const float* reg, float l_s, float* loss,
                          void* stream);
DV_API int dv_l2_loss_bwd(long long n, const float* x, const float* y, const float* grad, float l_s, float* dx,
                          float* dreg, void* stream);

/* Accumulates the feature-grid gradient (grad_voxels, same layout as voxels)
 * and the packed parameter gradient (grad_params) of the segments' decode. */
DV_API int dv_decode_bwd(int kind, int channels, const float* params, const float* voxels, int nvx,
                         int nvy, int nvz, const float* seg, const int* seg_ray, long long n_seg,
                         const int64_t* n_seg_dev, const float* pe_feat, const float* pe_out,
                         const float* d4, float* grad_voxels, float* grad_params, void* stream);

/*
 * Tensor-core form of dv_decode_fwd: the same decoder with its matrix
 * products on tcgen05 (BF16 when bf16 = 1, FP16 when 0, FP32 accumulation in
 * TMEM).  The integral, biases, PE term (pe_out, FP32), ReLU and sigmoid stay
 * in FP32.  wblob holds every layer's weight matrix [N][K] in the K-major
 * 8x8 core-matrix layout; `layers` is a HOST array of n_layers rows
 * (byte offset, K, N, bias offset); bias [nbias] floats.  err (device int,
 * optional) is set to 1 if a bounded wait for an MMA ran out.  voxels16
 * (optional, may be NULL): a copy of the grid in the operand format (BF16
 * when bf16 = 1, else FP16), same layout; when given, the corner rows are read
 * from it (half the bytes) and integrated in FP32.  save (optional, 16-byte
 * aligned, save_capacity bytes >= dv_decode_tc_save_bytes): receives the
 * layer inputs for dv_decode_bwd_tc.
 */
DV_API int dv_decode_fwd_tc(int kind, int channels, int bf16, const void* wblob, int wbytes,
                            const float* bias, int nbias, const int* layers, int n_layers,
                            const float* voxels, const void* voxels16, int nvx, int nvy, int nvz,
                            const float* seg, const int* seg_ray, long long n_seg,
                            const int64_t* n_seg_dev, const float* pe_out, float* out4, void* save,
                            long long save_capacity, int* err, void* stream);

/* Self-test of the bounded completion waits of the tensor-core kernels (no
 * counterpart in the reference): status (device int[2]) gets status[0] = 1
 * when a wait on an mbarrier that nobody arrives on gave up after `limit`
 * polls (at most 2^20), status[1] = 0 when a wait after an arrival completed.
 * The kernels report such a timeout through their `err` word and stop
 * issuing work; nothing spins unbounded. */
DV_API int dv_wait_selftest(int limit, int* status, void* stream);

/* Bytes of the `save` buffer of dv_decode_fwd_tc for n_seg segments: per
 * tile of 128 segments, every layer's input tile (BF16/FP16, the K-major
 * operand layout) in layer order; dv_decode_bwd_tc reads them back instead
 * of gathering the corner rows and recomputing the forward.  No counterpart
 * in the reference (its backward is torch autograd over stored activations). */
DV_API long long dv_decode_tc_save_bytes(int kind, int channels, long long n_seg);

/*
 * Split-operand form of dv_decode_fwd_tc (no counterpart in the reference,
 * whose decoder runs FP32 torch GEMMs): FP32-grade products on BF16 tensor
 * cores.  Every FP32 operand (the integrated features, each layer's
 * activations, the weights) is carried as three BF16 terms, each rounding what
 * the previous ones left, and each layer sums the six products whose term
 * indices add up to at most 2 in FP32 accumulators (about 2^-24 relative per
 * product).  wblob holds three terms of the images of dv_decode_fwd_tc, one
 * after the other, wbytes apart (wbytes = one term's bytes); `layers`, bias and
 * the rest as dv_decode_fwd_tc; the corner rows come from the FP32 grid.  save
 * (optional, >= dv_decode_tc_split_save_bytes): receives every layer input as
 * two BF16 terms for dv_decode_bwd_tc_split: per tile of 128 segments and
 * layer, one [128][2K] K-major core-matrix tile (256 * 2K bytes) with term j
 * in columns jK..jK+K-1.
 */
DV_API int dv_decode_fwd_tc_split(int kind, int channels, const void* wblob, int wbytes,
                                  const float* bias, int nbias, const int* layers, int n_layers,
                                  const float* voxels, int nvx, int nvy, int nvz, const float* seg,
                                  const int* seg_ray, long long n_seg, const int64_t* n_seg_dev,
                                  const float* pe_out, float* out4, void* save,
                                  long long save_capacity, int* err, void* stream);

/* Bytes of the `save` buffer of dv_decode_fwd_tc_split for n_seg segments:
 * per tile of 128 segments, every layer input tile as two BF16 terms. */
DV_API long long dv_decode_tc_split_save_bytes(int kind, int channels, long long n_seg);

/*
 * Weight image gather (no counterpart in the reference, whose decoder reads
 * the FP32 parameters directly): out[i] = ext[index[i]] with ext[0] = 0 and
 * ext[j] = params[j - 1], converted by form: 0 FP32, 1 BF16, 2 FP16, 3 three
 * BF16 terms (term t, the round-to-nearest-even of what terms 0..t-1 left, at
 * out + t * n * 2 bytes).  One launch rebuilds a tensor-core weight image (or
 * the bias vector) from the packed plain parameters after an optimizer step;
 * indices outside 0..n_params read 0.
 */
DV_API int dv_tc_image(const float* params, long long n_params, const int64_t* index, long long n,
                       int form, void* out, void* stream);

/*
 * Allocation-free form of dv_exclusive_scan (no counterpart in the reference,
 * which allocates all its buffers with torch).  For callers that cannot
 * allocate device memory themselves — an embedding host whose allocator owns
 * the device, a frame loop with a fixed memory budget, code running while a
 * CUDA graph is captured.  The tile sums live in a 32 KiB array inside the
 * library (present on every device that loads it, until the process exits).
 * n may be at most dv_exclusive_scan_static_max() (8,388,608 counts); larger
 * n returns DV_ERR_OVERFLOW without launching anything.  The first call on a
 * device with n > 0 looks up the array's address (once per device, with that
 * device current): make it before any stream capture.  The address stays
 * cached for the process, so the entry point must not be used on a device
 * after cudaDeviceReset.  Calls share the array, so calls that overlap on the
 * GPU race and must be serialised by the caller.  Calls no cudaMalloc/cudaFree.
 */
DV_API long long dv_exclusive_scan_static_max(void);
DV_API int dv_exclusive_scan_static(const int* counts, long long n, int64_t* offsets, void* stream);

/*
 * Tensor-core form of dv_decode_bwd (DIVeR32, 32 channels): recomputes the
 * forward on tcgen05 with the images of dv_decode_fwd_tc (wf, f_layers rows
 * of 4 ints), propagates deltas through wb, the transposed weights
 * [N = in][K = out padded to 16] per layer (b_layers: HOST rows of
 * (byte offset, K, N)); weight gradients accumulate in FP32 from BF16/FP16
 * activations and deltas.  Returns DV_ERR_UNSUPPORTED for other decoders.
 * saved (optional, with saved_bytes and the forward's out4): the save buffer
 * that dv_decode_fwd_tc filled for the same segments and weights; the
 * forward is then read back instead of recomputed (same bits).
 */
DV_API int dv_decode_bwd_tc(int kind, int channels, int bf16, const void* wf, int wf_bytes,
                            const float* bias, int nbias, const int* f_layers, const void* wb,
                            int wb_bytes, const int* b_layers, int n_layers, const float* voxels,
                            int nvx, int nvy, int nvz, const float* seg, const int* seg_ray,
                            long long n_seg, const int64_t* n_seg_dev, const float* pe_feat,
                            const float* pe_out, const float* d4, const void* saved,
                            long long saved_bytes, const float* out4, float* grad_voxels,
                            float* grad_params, int* err, void* stream);

/*
 * Split-operand form of dv_decode_bwd_tc (DIVeR32, 32 channels; no
 * counterpart in the reference): FP32-grade gradients on BF16 tensor cores.
 * Deltas propagate through three BF16 terms of each transposed weight image
 * (wb: three terms of dv_decode_bwd_tc's images, wb_term_bytes apart;
 * b_layers: HOST rows of (byte offset inside a term, K, N)) with six products
 * per layer; weight and bias gradients accumulate in FP32 from two-term deltas
 * and activations (all four products).  saved: the record dv_decode_fwd_tc_split
 * wrote for the same segments and weights (saved_bytes >=
 * dv_decode_tc_split_save_bytes), out4 its output; the forward is read back,
 * never recomputed.  Adds into grad_voxels and grad_params like dv_decode_bwd.
 * touched (optional, a byte per grid row): set at each segment's lower corner,
 * as dv_mark_corner_rows does, so no separate marking launch is needed.
 */
DV_API int dv_decode_bwd_tc_split(int kind, int channels, const void* wb, int wb_term_bytes,
                                  const int* b_layers, int n_layers, int nvx, int nvy, int nvz,
                                  const float* seg, const int* seg_ray, long long n_seg,
                                  const int64_t* n_seg_dev, const float* pe_feat, const float* d4,
                                  const void* saved, long long saved_bytes, const float* out4,
                                  float* grad_voxels, float* grad_params, unsigned char* touched, int* err, void* stream);

/* Clearing a grid gradient where a step wrote it (no counterpart in the
 * reference, whose optimizer zeroes the whole dense gradient every step).
 * touched: a byte per grid row (nvz * nvy * nvx, zero-initialised).
 * dv_mark_corner_rows sets the byte of the lower corner (as the integration
 * computes it) of each of the n_seg segments seg [n_seg][6] (n_seg_dev, when
 * not null, a device count <= n_seg of the valid ones).  dv_clear_marked_rows
 * zeroes every row of grid [nvz][nvy][nvx][channels] that is one of the 8
 * corners of a marked cell, then zeroes touched.  Marking a step's segments
 * after clearing and before its gradient scatter keeps the buffer zero
 * everywhere the next step does not write. */
DV_API int dv_mark_corner_rows(const float* seg, long long n_seg, const int64_t* n_seg_dev, int nvx,
                               int nvy, int nvz, uint8_t* touched, void* stream);
DV_API int dv_clear_marked_rows(float* grid, int channels, int nvx, int nvy, int nvz, uint8_t* touched,
                                void* stream);

/* Pinhole camera rays of pixels [first_pixel, first_pixel + n_pixels) of an
 * H x W image, row-major (utils/dataset/ray_utils.py:5-55): rays_o / rays_d
 * [n_pixels][3] (device); c2w is a HOST float [3][4] camera-to-world matrix;
 * directions unit length. */
DV_API int dv_camera_rays(int H, int W, float focal, const float* c2w, long long first_pixel,
                          long long n_pixels, float* rays_o, float* rays_d, void* stream);

/* ------------------------------------------------------------------------
 * Real-time path: occupancy-octree first hit and 8-hit ray march.
 * ------------------------------------------------------------------------ */

/*
 * First occupied 4^3 block of each pixel's ray through three max-pooled
 * occupancy levels (N/64, N/16, N/4).  Replaces aabb_intersect_wrapper
 *   (utils/ray_march/src/ray_march.cu:237-266) and aabb_intersect_kernel
 *   (same file :24-149).
 *   coords   [8][batch][6] hit buffer; slot 7 [3:6] receives the resume point
 *            (x = -1 on a miss)
 *   v        [batch][3] unit directions
 *   center   [3] camera centre in voxel units (device pointer)
 *   finish   [batch] bytes; set to 1 on a miss, else 0
 *   rgba     [batch][4]; initialised to (0,0,0,1)
 *   octrees  bytes, levels (N/64)^3, (N/16)^3, (N/4)^3 concatenated
 *   voxel_num  N, a multiple of 64
 */
DV_API int dv_aabb_intersect(int batch_size, float* coords, const float* v, const float* center,
                      uint8_t* finish, float* rgba, const uint8_t* octrees, int voxel_num,
                      void* stream);

/*
 * Records the next (up to) 8 occupied voxels of every unfinished ray into
 * coords[hit][b][0:6], resuming from coords[7][b][3:6]; a ray that leaves the
 * grid gets x = -1 in the slot after its last hit.  Replaces ray_march_wrapper
 *   (utils/ray_march/src/ray_march.cu:268-296) and ray_march_kernel (:151-230).
 *   mask  [N][N][N] occupancy bytes
 */
DV_API int dv_ray_march(int batch_size, float* coords, const float* v, const uint8_t* mask,
                 const uint8_t* finish, int voxel_num, void* stream);

/* ------------------------------------------------------------------------
 * Real-time fused decoder (per pixel, up to 8 hits per call).
 * ------------------------------------------------------------------------ */

/* Floats of the aligned weight layout for width 32 (DIVeR32) or 64 (DIVeR64). */
DV_API int dv_realtime_packed_size(int width);

/*
 * Re-lays out the reference's flat `params` array (convert.py:94-140; 3168
 * floats for DIVeR32, 8288 for DIVeR64, device memory) into the aligned
 * layout dv_mlp_eval reads.  Together with keeping the voxel map as a
 * caller-owned device buffer this replaces upload_weight_wrapper
 * (utils/mlp_evaluation/src/mlp_eval.cu:264-295), which binds a process-global
 * texture and __constant__ array.
 */
DV_API int dv_realtime_pack(int width, const float* ref_params, float* packed, void* stream);

/*
 * One round of the real-time decoder for every unfinished pixel: up to 8 hits
 * from coords [8][batch][6], feature table voxels [F][32], corner index map
 * voxel_map [map_size^3] (clamped lookups), packed weights, directions v
 * [batch][3]; updates rgba [batch][4] and finish [batch] in place.
 * Replaces mlp_eval_wrapper + mlp_eval_kernel
 * (utils/mlp_evaluation/src/mlp_eval.cu:32-254, width 32;
 *  utils/mlp_evaluation64/src/mlp_eval.cu:32-254, width 64).
 */
DV_API int dv_mlp_eval(int width, int batch_size, const float* coords, const float* voxels,
                       const int* voxel_map, int map_size, const float* packed_params, const float* v,
                       float* rgba, uint8_t* finish, void* stream);

/*
 * Tensor-core form of dv_mlp_eval (same contract: rgba and finish in place,
 * coords [8][B][6], the sparse feature table, the index map, the aligned
 * params of dv_realtime_pack), replacing the per-pixel FP32 layer loops of the
 * reference kernel (utils/mlp_evaluation{,64}/src/mlp_eval.cu:125-209) with
 * tcgen05 MMAs over tiles of 128 pixels, one tile per hit slot.  Operands
 * are split BF16 (three terms, six products per layer), so the results are
 * FP32-grade.  tc_blob: dv_realtime_tc_bytes(width) bytes (16-byte aligned)
 * filled once per model by dv_realtime_tc_pack from the same aligned params.
 * err (device int, optional): set to 1 if a bounded MMA completion wait ran
 * out.
 */
DV_API int dv_realtime_tc_bytes(int width);
DV_API int dv_realtime_tc_pack(int width, const float* packed_params, void* tc_blob, void* stream);
DV_API int dv_mlp_eval_tc(int width, int batch_size, const float* coords, const float* voxels,
                          const int* voxel_map, int map_size, const float* packed_params,
                          const void* tc_blob, const float* v, float* rgba, uint8_t* finish, int* err,
                          void* stream);

/*
 * Whole real-time frame in one launch (no counterpart call in the reference,
 * whose eval_rt.py:115-122 loops on the host: dv_aabb_intersect, then rounds
 * of dv_ray_march + dv_mlp_eval until every pixel is finished).  Per pixel:
 * the octree first hit, then the fine-grid walk, each occupied voxel decoded
 * as it is reached, until the ray leaves the grid or T < 1e-2.  Same per-pixel
 * arithmetic and order as the host loop, so rgba [batch][4] (rgb, T) equals
 * its result; center is the camera centre in voxel units (device [3]);
 * octrees / voxel_mask / voxels / voxel_map / packed_params as for
 * dv_aabb_intersect, dv_ray_march and dv_mlp_eval (map_size = N + 1).
 */
DV_API int dv_realtime_frame(int width, int batch_size, const float* v, const float* center,
                             const uint8_t* octrees, int N, const uint8_t* voxel_mask,
                             const float* voxels, const int* voxel_map, int map_size,
                             const float* packed_params, float* rgba, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* DIVER_GB300_H */
