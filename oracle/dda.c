/*
 * ORACLE — test infrastructure only.  CPU restatement of the DIVeR reference
 * traversal kernels, used by tests/ and by bench.py's CPU baseline as the
 * checker; never linked into or called by the product library.
 *
 * Parity pin: the outputs of these functions are compared in tests/ with
 * fixtures produced by the reference's own CUDA kernels
 * (tests/golden/traverse_ref.npz, generated by oracle/ref_kernels.py).
 *
 * Build with -ffp-contract=off: every multiply and add below rounds on its
 * own, and the one contraction the reference's compiler performs
 * (the position update ori + dir*t under nvcc's default -fmad=true) is written
 * as fmaf().  The `fused` flag switches that update to a separate multiply and
 * add, which is how the fixtures show which of the two the reference used.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

typedef struct { float x, y, z; } v3;

/* Walks that stopped at their step bound (see walk_cap). */
static long long cap_hits = 0;

/* A direction with a non-finite component, or a zero direction, does not
 * advance one grid plane per step (its steps are NaN or -inf and the walk
 * would never leave the grid): such a ray is a miss.  The reference kernels
 * have no such check and loop forever on it. */
static int dir_ok(v3 d) {
  return isfinite(d.x) && isfinite(d.y) && isfinite(d.z) && (d.x != 0.f || d.y != 0.f || d.z != 0.f);
}

/* Step bound of a walk through a box of nx x ny x nz cells: every step snaps
 * one axis onto its next grid plane and the coordinates move monotonically,
 * so a ray crosses at most n + 1 planes per axis before it leaves. */
static int walk_cap(float nx, float ny, float nz) { return (int)(nx + ny + nz) + 3; }

long long oracle_walk_cap_hits(int reset) {
  long long v = cap_hits;
  if (reset) cap_hits = 0;
  return v;
}

static float sgnf(float x) { return x > 0.f ? 1.f : (x < 0.f ? -1.f : 0.f); }
static float clampf(float v, float lo, float hi) { return fmaxf(lo, fminf(v, hi)); }
static float madd(float a, float b, float c, int fused) {
  if (fused) return fmaf(a, b, c);
  volatile float p = a * b;
  return p + c;
}

/* Slab test: utils/ray_voxel_intersection/src/ray_voxel_intersect.cu:61-100,
 * utils/ray_march/src/ray_march.cu:58-88. */
static int box_entry(v3* p, v3 d, float n, float* t, int fused) {
  int inside = (p->x >= 0.f) & (p->y >= 0.f) & (p->z >= 0.f) & (p->x <= n) & (p->y <= n) & (p->z <= n);
  if (inside) {
    *t = 0.f;
    return 1;
  }
  float a = (-p->x) / d.x, b = (n - p->x) / d.x;
  float lo = fminf(a, b), hi = fmaxf(a, b);
  a = (-p->y) / d.y;
  b = (n - p->y) / d.y;
  lo = fmaxf(lo, fminf(a, b));
  hi = fminf(hi, fmaxf(a, b));
  a = (-p->z) / d.z;
  b = (n - p->z) / d.z;
  lo = fmaxf(lo, fminf(a, b));
  hi = fminf(hi, fmaxf(a, b));
  p->x = clampf(madd(d.x, lo, p->x, fused), 0.f, n);
  p->y = clampf(madd(d.y, lo, p->y, fused), 0.f, n);
  p->z = clampf(madd(d.z, lo, p->z, fused), 0.f, n);
  *t = lo;
  return !(lo > hi);
}

/* One DDA step: ray_voxel_intersect.cu:119-135. */
static v3 grid_step(v3 a, v3 d, v3 s, float* dt, int fused) {
  float bx = floorf(a.x * s.x + 1.f) * s.x;
  float by = floorf(a.y * s.y + 1.f) * s.y;
  float bz = floorf(a.z * s.z + 1.f) * s.z;
  float tx = (bx - a.x) / d.x, ty = (by - a.y) / d.y, tz = (bz - a.z) / d.z;
  float t = fminf(tx, fminf(ty, tz));
  v3 b;
  b.x = madd(d.x, t, a.x, fused);
  b.y = madd(d.y, t, a.y, fused);
  b.z = madd(d.z, t, a.z, fused);
  if (t == tx) b.x = bx;
  else if (t == ty) b.y = by;
  else b.z = bz;
  *dt = t;
  return b;
}

static int out_closed(v3 b, float n) {
  return (b.x < 0.f) | (b.y < 0.f) | (b.z < 0.f) | (b.x > n) | (b.y > n) | (b.z > n);
}
static int out_open(v3 b, float n) {
  return (b.x < 0.f) | (b.y < 0.f) | (b.z < 0.f) | (b.x >= n) | (b.y >= n) | (b.z >= n);
}

/* ray_voxel_intersect.cu:297-299 (and ray_march.cu:132-135 with scale 1). */
static long long cell(v3 a, v3 b, float scale, int m) {
  float cx = fminf(a.x + 1e-4f, b.x + 1e-4f) * scale;
  float cy = fminf(a.y + 1e-4f, b.y + 1e-4f) * scale;
  float cz = fminf(a.z + 1e-4f, b.z + 1e-4f) * scale;
  return (long long)(int)cz * m * m + (long long)(int)cy * m + (int)cx;
}

static int occ(const uint8_t* mask, long long idx, long long cells) {
  return (idx >= 0 && idx < cells) ? mask[idx] != 0 : 0;
}

/* ray_voxel_intersect_kernel, ray_voxel_intersect.cu:29-151.  Buffers follow
 * the reference wrapper: intersection zero-filled [B][max_n][3], tns filled
 * with -1 [B][max_n]; num written.  Points past max_n are counted only. */
void oracle_dense_walk(int batch, int max_n, float xyzmin, float n, float vs, const float* o,
                       const float* v, float* inter, int* num, float* tns, int fused) {
  for (int b = 0; b < batch; ++b) {
    v3 d = {v[3 * b], v[3 * b + 1], v[3 * b + 2]};
    v3 p = {(o[3 * b] - xyzmin) / vs, (o[3 * b + 1] - xyzmin) / vs, (o[3 * b + 2] - xyzmin) / vs};
    float t;
    int hit = dir_ok(d) && box_entry(&p, d, n, &t, fused);
    float* row = inter + (long long)b * max_n * 3;
    float* trow = tns + (long long)b * max_n;
    int count = 0;
    if (max_n > 0) {
      row[0] = p.x;
      row[1] = p.y;
      row[2] = p.z;
    }
    if (hit) {
      if (max_n > 0) trow[0] = t * vs;
      count = 1;
      v3 s = {sgnf(d.x), sgnf(d.y), sgnf(d.z)};
      const int cap = walk_cap(n, n, n);
      int k = 0;
      for (; k < cap; ++k) {
        float dt;
        v3 q = grid_step(p, d, s, &dt, fused);
        t = t + dt;
        if (out_closed(q, n)) break;
        if (count < max_n) {
          row[3 * count] = q.x;
          row[3 * count + 1] = q.y;
          row[3 * count + 2] = q.z;
          trow[count] = t * vs;
        }
        ++count;
        p = q;
      }
      if (k == cap) ++cap_hits;
    }
    num[b] = count;
  }
}

/* masked_intersect_kernel, ray_voxel_intersect.cu:192-319. */
void oracle_masked_walk(int batch, int max_n, float xyzmin, float n, float vs, float mask_scale,
                        const float* o, const float* v, const uint8_t* mask, float* inter, int* num,
                        float* tns, int fused) {
  volatile float mprod = n * mask_scale;
  int m = (int)mprod;
  long long cells = (long long)m * m * m;
  for (int b = 0; b < batch; ++b) {
    v3 d = {v[3 * b], v[3 * b + 1], v[3 * b + 2]};
    v3 p = {(o[3 * b] - xyzmin) / vs, (o[3 * b + 1] - xyzmin) / vs, (o[3 * b + 2] - xyzmin) / vs};
    float t;
    int count = 0;
    if (dir_ok(d) && box_entry(&p, d, n, &t, fused)) {
      v3 s = {sgnf(d.x), sgnf(d.y), sgnf(d.z)};
      float* row = inter + (long long)b * max_n * 6;
      float* trow = tns + (long long)b * max_n;
      const int cap = walk_cap(n, n, n);
      int k = 0;
      for (; k < cap; ++k) {
        float dt;
        v3 q = grid_step(p, d, s, &dt, fused);
        t = t + dt;
        if (out_closed(q, n)) break;
        if (occ(mask, cell(p, q, mask_scale, m), cells)) {
          if (count < max_n) {
            float* r = row + 6 * count;
            r[0] = p.x; r[1] = p.y; r[2] = p.z;
            r[3] = q.x; r[4] = q.y; r[5] = q.z;
            trow[count] = t * vs;
          }
          ++count;
        }
        p = q;
      }
      if (k == cap) ++cap_hits;
    }
    num[b] = count;
  }
}

/* aabb_intersect_kernel, ray_march.cu:24-149, for any N multiple of 64. */
void oracle_aabb(int batch, float* coords, const float* v, const float* center, uint8_t* finish,
                 float* rgba, const uint8_t* oct, int N, int fused) {
  long long l0 = N / 64, l1 = N / 16, l2 = N / 4;
  long long cells = l0 * l0 * l0 + l1 * l1 * l1 + l2 * l2 * l2;
  for (int b = 0; b < batch; ++b) {
    float* slot = coords + (long long)batch * 6 * 7 + (long long)b * 6 + 3;
    rgba[4 * b] = rgba[4 * b + 1] = rgba[4 * b + 2] = 0.f;
    rgba[4 * b + 3] = 1.f;
    finish[b] = 0;
    v3 d = {v[3 * b], v[3 * b + 1], v[3 * b + 2]};
    v3 p = {center[0], center[1], center[2]};
    float t;
    if (!dir_ok(d) || !box_entry(&p, d, (float)N, &t, fused)) {
      slot[0] = -1.f;
      finish[b] = 1;
      continue;
    }
    p.x /= 64.f; p.y /= 64.f; p.z /= 64.f;
    v3 s = {sgnf(d.x), sgnf(d.y), sgnf(d.z)};
    int m = N / 64;
    long long off = 0;
    v3 last = p;
    int missed = 0;
    /* every level walks fewer than 3 (N / 4) + 3 steps */
    const int cap = walk_cap((float)N, 0.f, 0.f) + 6;
    int steps = 0;
    while (m < N) {
      if (steps++ == cap) {
        ++cap_hits;
        slot[0] = -1.f;
        finish[b] = 1;
        missed = 1;
        break;
      }
      last = p;
      float dt;
      v3 q = grid_step(last, d, s, &dt, fused);
      if (out_closed(q, (float)m)) {
        slot[0] = -1.f;
        finish[b] = 1;
        missed = 1;
        break;
      }
      if (occ(oct, off + cell(last, q, 1.f, m), cells)) {
        off += (long long)m * m * m;
        last.x *= 4.f; last.y *= 4.f; last.z *= 4.f;
        p = last;
        m *= 4;
      } else {
        p = q;
      }
    }
    if (!missed) {
      slot[0] = last.x;
      slot[1] = last.y;
      slot[2] = last.z;
    }
  }
}

/* ray_march_kernel, ray_march.cu:151-230 (per ray; see the kernel comment
 * about the unreachable resume-point check). */
void oracle_ray_march(int batch, float* coords, const float* v, const uint8_t* mask,
                      const uint8_t* finish, int N, int fused) {
  long long stride = (long long)batch * 6;
  long long cells = (long long)N * N * N;
  for (int b = 0; b < batch; ++b) {
    if (finish[b]) continue;
    const float* rs = coords + 7 * stride + (long long)b * 6 + 3;
    v3 last = {rs[0], rs[1], rs[2]};
    coords[(long long)b * 6] = -1.f;
    if (last.x < 0.f) continue;
    v3 d = {v[3 * b], v[3 * b + 1], v[3 * b + 2]};
    if (!dir_ok(d)) continue;
    v3 s = {sgnf(d.x), sgnf(d.y), sgnf(d.z)};
    int hits = 0;
    const int cap = walk_cap((float)N, (float)N, (float)N);
    int steps = 0;
    while (hits < 8) {
      if (steps++ == cap) {
        ++cap_hits;
        coords[hits * stride + (long long)b * 6] = -1.f;
        break;
      }
      float dt;
      v3 q = grid_step(last, d, s, &dt, fused);
      if (out_open(q, (float)N)) {
        coords[hits * stride + (long long)b * 6] = -1.f;
        break;
      }
      if (occ(mask, cell(last, q, 1.f, N), cells)) {
        float* r = coords + hits * stride + (long long)b * 6;
        r[0] = last.x; r[1] = last.y; r[2] = last.z;
        r[3] = q.x; r[4] = q.y; r[5] = q.z;
        ++hits;
      }
      last = q;
    }
  }
}

/* Masked walk over a grid with per-axis extents dims[3] (nx, ny, nz) and
 * origin xyzmin[3]: the same walk as oracle_masked_walk with the box
 * [0,nx]x[0,ny]x[0,nz], occupancy [nz][ny][nx], mask scale 1. */
void oracle_masked_walk_grid(int batch, int max_n, const float* xyzmin, const int* dims, float vs, const float* o,
                             const float* v, const uint8_t* mask, float* inter, int* num, float* tns) {
  float nx = (float)dims[0], ny = (float)dims[1], nz = (float)dims[2];
  long long cells = (long long)dims[0] * dims[1] * dims[2];
  for (int b = 0; b < batch; ++b) {
    v3 d = {v[3 * b], v[3 * b + 1], v[3 * b + 2]};
    v3 p = {(o[3 * b] - xyzmin[0]) / vs, (o[3 * b + 1] - xyzmin[1]) / vs, (o[3 * b + 2] - xyzmin[2]) / vs};
    float t = 0.f;
    int count = 0, hit = dir_ok(d);
    int inside = (p.x >= 0.f) & (p.y >= 0.f) & (p.z >= 0.f) & (p.x <= nx) & (p.y <= ny) & (p.z <= nz);
    if (hit && !inside) {
      float a = (-p.x) / d.x, c = (nx - p.x) / d.x;
      float lo = fminf(a, c), hi = fmaxf(a, c);
      a = (-p.y) / d.y; c = (ny - p.y) / d.y;
      lo = fmaxf(lo, fminf(a, c)); hi = fminf(hi, fmaxf(a, c));
      a = (-p.z) / d.z; c = (nz - p.z) / d.z;
      lo = fmaxf(lo, fminf(a, c)); hi = fminf(hi, fmaxf(a, c));
      p.x = clampf(fmaf(d.x, lo, p.x), 0.f, nx);
      p.y = clampf(fmaf(d.y, lo, p.y), 0.f, ny);
      p.z = clampf(fmaf(d.z, lo, p.z), 0.f, nz);
      t = lo;
      hit = !(lo > hi);
    }
    if (hit) {
      v3 s = {sgnf(d.x), sgnf(d.y), sgnf(d.z)};
      float* row = inter + (long long)b * max_n * 6;
      float* trow = tns + (long long)b * max_n;
      const int cap = walk_cap(nx, ny, nz);
      int k = 0;
      for (; k < cap; ++k) {
        float dt;
        v3 q = grid_step(p, d, s, &dt, 1);
        t = t + dt;
        if ((q.x < 0.f) | (q.y < 0.f) | (q.z < 0.f) | (q.x > nx) | (q.y > ny) | (q.z > nz)) break;
        float cx = fminf(p.x + 1e-4f, q.x + 1e-4f), cy = fminf(p.y + 1e-4f, q.y + 1e-4f),
              cz = fminf(p.z + 1e-4f, q.z + 1e-4f);
        long long idx = ((long long)(int)cz * dims[1] + (int)cy) * dims[0] + (int)cx;
        if (occ(mask, idx, cells)) {
          if (count < max_n) {
            float* r = row + 6 * count;
            r[0] = p.x; r[1] = p.y; r[2] = p.z;
            r[3] = q.x; r[4] = q.y; r[5] = q.z;
            trow[count] = t * vs;
          }
          ++count;
        }
        p = q;
      }
      if (k == cap) ++cap_hits;
    }
    num[b] = count;
  }
}
