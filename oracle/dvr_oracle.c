/*
 * DiffDVR ray-marcher oracle — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's forward and adjoint volume ray
 * marcher, written from the published algorithm and checked against the
 * reference's own CPU templates (oracle/ref_harness.cpp) and the golden
 * fixtures in tests/golden/.  It is the checker for the CUDA kernels in
 * diffdvr_gb300 and the "port" CPU baseline; the product never calls it.
 *
 * Built twice: DVR_ORACLE_DOUBLE=1 (real_t = double, the FP64 oracle) and
 * DVR_ORACLE_DOUBLE=0 (real_t = float, which follows the reference's FP32 CPU
 * build operation for operation).  Parallel over rays with OpenMP; every
 * gradient scatter is an `omp atomic`, as in renderer/renderer_adjoint.cuh:16-26.
 *
 * Citations are to files of the reference project (shamanDevel/DiffDVR).
 */
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include <stddef.h>
#include <stdlib.h>
#include <string.h>

#if DVR_ORACLE_DOUBLE
typedef double real_t;
#define R_EXP exp
#define R_SQRT sqrt
#define R_TAN tan
#define R_ROUND round
#define R_FMIN fmin
#define R_FMAX fmax
#else
typedef float real_t;
#define R_EXP expf
#define R_SQRT sqrtf
#define R_TAN tanf
#define R_ROUND roundf
#define R_FMIN fminf
#define R_FMAX fmaxf
#endif

/* real_t is this build's; the header declares the per-step components with it */
#define DVR_ORACLE_HAS_REAL_T 1
#include "dvr_oracle.h"

typedef struct { real_t x, y, z; } v3;
typedef struct { real_t x, y, z, w; } v4;

/* ---- small vector helpers (same operation order as the reference's helper
 *      math: dot = x*x' + y*y' + z*z' [+ w*w'], lerp(a,b,t) = a + t*(b-a)) ---- */
static inline v3 mk3(real_t x, real_t y, real_t z) { v3 r = {x, y, z}; return r; }
static inline v4 mk4(real_t x, real_t y, real_t z, real_t w) { v4 r = {x, y, z, w}; return r; }
static inline real_t dot3(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline real_t dot4(v4 a, v4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
static inline real_t lerp1(real_t a, real_t b, real_t t) { return a + t * (b - a); }
static inline real_t rmin(real_t a, real_t b) { return a < b ? a : b; }
static inline real_t rmax(real_t a, real_t b) { return a > b ? a : b; }
static inline real_t clampr(real_t v, real_t lo, real_t hi) { return R_FMAX(lo, R_FMIN(v, hi)); }
static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
static inline v3 cross3(v3 a, v3 b) {
  return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline v3 normalize3(v3 v) {
  /* host-side rsqrt is 1/sqrt (renderer/helper_math.cuh:74-82) */
  real_t inv = (real_t)1 / R_SQRT(dot3(v, v));
  return mk3(v.x * inv, v.y * inv, v.z * inv);
}

/* ---- broadcasting strided access (renderer/renderer_tensor.cuh:140-144) ---- */
static inline int64_t bstride(const OracleTensor* t, int d) { return t->sizes[d] == 1 ? 0 : t->strides[d]; }
static inline real_t* at2(const OracleTensor* t, int64_t i0, int64_t i1) {
  return (real_t*)t->data + i0 * bstride(t, 0) + i1 * bstride(t, 1);
}
static inline real_t* at3(const OracleTensor* t, int64_t i0, int64_t i1, int64_t i2) {
  return (real_t*)t->data + i0 * bstride(t, 0) + i1 * bstride(t, 1) + i2 * bstride(t, 2);
}
static inline real_t* at4(const OracleTensor* t, int64_t i0, int64_t i1, int64_t i2, int64_t i3) {
  return (real_t*)t->data + i0 * bstride(t, 0) + i1 * bstride(t, 1) + i2 * bstride(t, 2) + i3 * bstride(t, 3);
}
static inline int32_t* iat3(const OracleTensor* t, int64_t i0, int64_t i1, int64_t i2) {
  return (int32_t*)t->data + i0 * bstride(t, 0) + i1 * bstride(t, 1) + i2 * bstride(t, 2);
}
static inline void atomic_add(real_t* p, real_t v) {
#pragma omp atomic
  *p += v;
}

/* ---- camera (renderer/renderer_camera.cuh:13-59) ---- */
static void compute_ray(const OracleInputs* in, int x, int y, int b, v3* start, v3* dir) {
  if (in->camera_mode == 0) {
    const OracleTensor* s = &in->ray_start;
    const OracleTensor* d = &in->ray_dir;
    *start = mk3(*at4(s, b, y, x, 0), *at4(s, b, y, x, 1), *at4(s, b, y, x, 2));
    *dir = mk3(*at4(d, b, y, x, 0), *at4(d, b, y, x, 1), *at4(d, b, y, x, 2));
  } else if (in->camera_mode == 1) {
    /* unproject NDC (fx, fy) at depth 0 and 0.9 with the inverse view-projection
     * rows; matmul_proj divides by w (renderer/renderer_utils.cuh:43-58) */
    const OracleTensor* m = &in->camera_matrix;
    v4 row[4];
    for (int i = 0; i < 4; ++i)
      row[i] = mk4(*at3(m, b, i, 0), *at3(m, b, i, 1), *at3(m, b, i, 2), *at3(m, b, i, 3));
    const real_t fx = 2 * (x + (real_t)0.5) / (real_t)in->width - 1;
    const real_t fy = 2 * (y + (real_t)0.5) / (real_t)in->height - 1;
    v3 p[2];
    const real_t depth[2] = {0, (real_t)0.9};
    for (int k = 0; k < 2; ++k) {
      v4 s = mk4(fx, fy, depth[k], 1);
      v4 w = mk4(dot4(row[0], s), dot4(row[1], s), dot4(row[2], s), dot4(row[3], s));
      p[k] = mk3(w.x / w.w, w.y / w.w, w.z / w.w);
    }
    *start = p[0];
    *dir = normalize3(mk3(p[1].x - p[0].x, p[1].y - p[0].y, p[1].z - p[0].z));
  } else {
    /* reference frame: eye, right, up rows + vertical field of view */
    const OracleTensor* m = &in->camera_matrix;
    const real_t fovy = (real_t)in->fov_y_radians;
    const real_t fovx = fovy * (real_t)in->width / (real_t)in->height;
    const real_t tan_x = R_TAN(fovx / 2);
    const real_t tan_y = R_TAN(fovy / 2);
    v3 eye = mk3(*at3(m, b, 0, 0), *at3(m, b, 0, 1), *at3(m, b, 0, 2));
    v3 right = mk3(*at3(m, b, 1, 0), *at3(m, b, 1, 1), *at3(m, b, 1, 2));
    v3 up = mk3(*at3(m, b, 2, 0), *at3(m, b, 2, 1), *at3(m, b, 2, 2));
    v3 front = cross3(up, right);
    const real_t fx = 2 * (x + 0.5f) / (real_t)in->width - 1;
    const real_t fy = 2 * (y + 0.5f) / (real_t)in->height - 1;
    const real_t ax = fx * tan_x, ay = fy * tan_y;
    v3 d = mk3(front.x + ax * right.x + ay * up.x, front.y + ax * right.y + ay * up.y,
               front.z + ax * right.z + ay * up.z);
    *start = eye;
    *dir = normalize3(d);
  }
}

/* ---- slab test (renderer/renderer_utils.cuh:60-74) ---- */
static void ray_box(v3 s, v3 d, v3 bmin, v3 bsize, real_t* tmin, real_t* tmax) {
  const real_t ix = 1.0f / d.x, iy = 1.0f / d.y, iz = 1.0f / d.z;
  const real_t t1 = (bmin.x - s.x) * ix, t2 = (bmin.x + bsize.x - s.x) * ix;
  const real_t t3 = (bmin.y - s.y) * iy, t4 = (bmin.y + bsize.y - s.y) * iy;
  const real_t t5 = (bmin.z - s.z) * iz, t6 = (bmin.z + bsize.z - s.z) * iz;
  *tmin = rmax(rmax(rmin(t1, t2), rmin(t3, t4)), rmin(t5, t6));
  *tmax = rmin(rmin(rmax(t1, t2), rmax(t3, t4)), rmax(t5, t6));
}

/* ---- volume sampling (renderer/renderer_interpolation.cuh) ----
 * The per-ray cell cache of the reference (:187-240, :331-357) only avoids
 * refetches; results are those of a fresh fetch, so the oracle keeps a cache
 * only where it carries state: the adjoint's per-cell gradient accumulators. */
typedef struct {
  int b, X, Y, Z;
  const OracleTensor* vol;
  /* adjoint state */
  OracleTensor* adj;
  int has_adj;
  int li[3];          /* cell (trilinear) or voxel (nearest) of the accumulators */
  real_t dens[8];
  real_t acc[8];
  real_t fpos[3];
  real_t nearest_val, nearest_acc;
} Sampler;

static inline real_t vox(const Sampler* s, int x, int y, int z) { return *at4(s->vol, s->b, x, y, z); }

static void nearest_index(const Sampler* s, v3 p, int* ix) {
  /* clamp to [EPS, size-1-EPS] then round half away from zero (:36-49) */
  const real_t eps = (real_t)1e-7;
  const real_t one_eps = 1 + eps;
  ix[0] = (int)R_ROUND(clampr(p.x, eps, (real_t)s->X - one_eps));
  ix[1] = (int)R_ROUND(clampr(p.y, eps, (real_t)s->Y - one_eps));
  ix[2] = (int)R_ROUND(clampr(p.z, eps, (real_t)s->Z - one_eps));
}

static void cell_corners(const Sampler* s, const int* ip, real_t* d) {
  /* corner bit order zyx: bit2 = x high, bit1 = y high, bit0 = z high (:193-207) */
  const int lx = clampi(ip[0], 0, s->X - 1), hx = clampi(ip[0] + 1, 0, s->X - 1);
  const int ly = clampi(ip[1], 0, s->Y - 1), hy = clampi(ip[1] + 1, 0, s->Y - 1);
  const int lz = clampi(ip[2], 0, s->Z - 1), hz = clampi(ip[2] + 1, 0, s->Z - 1);
  d[0] = vox(s, lx, ly, lz); d[1] = vox(s, lx, ly, hz);
  d[2] = vox(s, lx, hy, lz); d[3] = vox(s, lx, hy, hz);
  d[4] = vox(s, hx, ly, lz); d[5] = vox(s, hx, ly, hz);
  d[6] = vox(s, hx, hy, lz); d[7] = vox(s, hx, hy, hz);
}

static real_t trilerp(const real_t* d, const real_t* f) {
  return lerp1(lerp1(lerp1(d[0], d[4], f[0]), lerp1(d[2], d[6], f[0]), f[1]),
               lerp1(lerp1(d[1], d[5], f[0]), lerp1(d[3], d[7], f[0]), f[1]), f[2]);
}

static real_t sample_forward(const Sampler* s, int filter, v3 p) {
  if (filter == 0) {
    int ix[3];
    nearest_index(s, p, ix);
    return vox(s, ix[0], ix[1], ix[2]);
  }
  /* truncation toward zero, not floor (:218) */
  int ip[3] = {(int)p.x, (int)p.y, (int)p.z};
  real_t d[8], f[3] = {p.x - (real_t)ip[0], p.y - (real_t)ip[1], p.z - (real_t)ip[2]};
  cell_corners(s, ip, d);
  return trilerp(d, f);
}

static void sampler_flush(Sampler* s, int filter) {
  if (!s->has_adj) return;
  if (filter == 0) {
    /* nearest: flush when the accumulated value is nonzero (:95-106) */
    if (s->nearest_acc != 0) {
      atomic_add(at4(s->adj, s->b, s->li[0], s->li[1], s->li[2]), s->nearest_acc);
      s->nearest_acc = 0;
    }
    return;
  }
  if (s->li[0] >= 0) { /* all eight corners, zero or not (:299-321) */
    const int lx = clampi(s->li[0], 0, s->X - 1), hx = clampi(s->li[0] + 1, 0, s->X - 1);
    const int ly = clampi(s->li[1], 0, s->Y - 1), hy = clampi(s->li[1] + 1, 0, s->Y - 1);
    const int lz = clampi(s->li[2], 0, s->Z - 1), hz = clampi(s->li[2] + 1, 0, s->Z - 1);
    atomic_add(at4(s->adj, s->b, lx, ly, lz), s->acc[0]);
    atomic_add(at4(s->adj, s->b, lx, ly, hz), s->acc[1]);
    atomic_add(at4(s->adj, s->b, lx, hy, lz), s->acc[2]);
    atomic_add(at4(s->adj, s->b, lx, hy, hz), s->acc[3]);
    atomic_add(at4(s->adj, s->b, hx, ly, lz), s->acc[4]);
    atomic_add(at4(s->adj, s->b, hx, ly, hz), s->acc[5]);
    atomic_add(at4(s->adj, s->b, hx, hy, lz), s->acc[6]);
    atomic_add(at4(s->adj, s->b, hx, hy, hz), s->acc[7]);
    for (int i = 0; i < 8; ++i) s->acc[i] = 0;
  }
}

/* fetch with adjoint state: switches cells (flushing the accumulators) */
static real_t sample_adjoint_fetch(Sampler* s, int filter, v3 p) {
  if (filter == 0) {
    int ix[3];
    nearest_index(s, p, ix);
    if (ix[0] != s->li[0] || ix[1] != s->li[1] || ix[2] != s->li[2]) {
      sampler_flush(s, filter);
      s->li[0] = ix[0]; s->li[1] = ix[1]; s->li[2] = ix[2];
      s->nearest_val = vox(s, ix[0], ix[1], ix[2]);
    }
    return s->nearest_val;
  }
  int ip[3] = {(int)p.x, (int)p.y, (int)p.z};
  if (ip[0] != s->li[0] || ip[1] != s->li[1] || ip[2] != s->li[2]) {
    sampler_flush(s, filter);
    s->li[0] = ip[0]; s->li[1] = ip[1]; s->li[2] = ip[2];
    cell_corners(s, ip, s->dens);
  }
  s->fpos[0] = p.x - (real_t)ip[0];
  s->fpos[1] = p.y - (real_t)ip[1];
  s->fpos[2] = p.z - (real_t)ip[2];
  return trilerp(s->dens, s->fpos);
}

/* adjoint of the trilinear weights (:360-387); returns d(density)/d(volumePos) * adj */
static v3 sample_adjoint(Sampler* s, int filter, real_t adj_density) {
  if (filter == 0) {
    s->nearest_acc += adj_density;
    return mk3(0, 0, 0);
  }
  const real_t c[3] = {s->fpos[0], s->fpos[1], s->fpos[2]};
  const real_t f[3] = {1 - c[0], 1 - c[1], 1 - c[2]};
  real_t adj_c[3] = {0, 0, 0}, adj_f[3] = {0, 0, 0};
  /* corner order of the reference's scatter list: 000,100,010,110,001,101,011,111 (xyz) */
  static const int order[8] = {0, 4, 2, 6, 1, 5, 3, 7};
  for (int k = 0; k < 8; ++k) {
    const int idx = order[k];
    const int hx = (idx >> 2) & 1, hy = (idx >> 1) & 1, hz = idx & 1;
    const real_t wx = hx ? c[0] : f[0], wy = hy ? c[1] : f[1], wz = hz ? c[2] : f[2];
    real_t* ax = hx ? &adj_c[0] : &adj_f[0];
    real_t* ay = hy ? &adj_c[1] : &adj_f[1];
    real_t* az = hz ? &adj_c[2] : &adj_f[2];
    if (s->has_adj) s->acc[idx] += adj_density * (wx * wy * wz);
    *ax += adj_density * s->dens[idx] * wy * wz;
    *ay += adj_density * s->dens[idx] * wx * wz;
    *az += adj_density * s->dens[idx] * wx * wy;
  }
  return mk3(adj_c[0] - adj_f[0], adj_c[1] - adj_f[1], adj_c[2] - adj_f[2]);
}

/* ---- transfer functions (renderer/renderer_tf.cuh) ---- */
static inline v4 tf4(const OracleTensor* tf, int b, int r) {
  return mk4(*at3(tf, b, r, 0), *at3(tf, b, r, 1), *at3(tf, b, r, 2), *at3(tf, b, r, 3));
}

static inline real_t gauss(real_t d, real_t mu, real_t sigma) {
  /* channel 5 is used as the standard deviation (:491-496) */
  return R_EXP(-(d - mu) * (d - mu) / (2 * sigma * sigma));
}

static int linear_interval(const OracleTensor* tf, int b, int R, real_t density) {
  /* the search stops at R-2 (:298-301) */
  int i;
  for (i = 0; i < R - 2; ++i)
    if (*at3(tf, b, i + 1, 4) > density) break;
  return i;
}

static v4 tf_eval(const OracleInputs* in, int b, real_t density) {
  const OracleTensor* tf = &in->tf;
  const int R = (int)tf->sizes[1];
  switch (in->tf_mode) {
    case 0: { /* identity: [0][0] absorption scale, [0][1] colour scale (:62-73) */
      const real_t d = clampr(density, 0, 1);
      const real_t sa = *at3(tf, b, 0, 0), sc = *at3(tf, b, 0, 1);
      return mk4(d * sc, d * sc, d * sc, d * sa);
    }
    case 1: { /* 1D texture, texel centres at (i+0.5)/R (:160-171) */
      const real_t d = density * R - (real_t)0.5;
      const int di = (int)floorf((float)d);
      const real_t df = d - di;
      const v4 a = tf4(tf, b, clampi(di, 0, R - 1)), c = tf4(tf, b, clampi(di + 1, 0, R - 1));
      return mk4(lerp1(a.x, c.x, df), lerp1(a.y, c.y, df), lerp1(a.z, c.z, df), lerp1(a.w, c.w, df));
    }
    case 2: { /* piecewise linear (:294-313) */
      const int i = linear_interval(tf, b, R, density);
      const v4 a = tf4(tf, b, i), c = tf4(tf, b, i + 1);
      const real_t p0 = *at3(tf, b, i, 4), p1 = *at3(tf, b, i + 1, 4);
      const real_t d = clampr(density, p0, p1);
      const real_t fr = (d - p0) / (p1 - p0);
      return mk4(lerp1(a.x, c.x, fr), lerp1(a.y, c.y, fr), lerp1(a.z, c.z, fr), lerp1(a.w, c.w, fr));
    }
    default: { /* sum of Gaussians (:507-519) */
      v4 acc = mk4(0, 0, 0, 0);
      for (int i = 0; i < R; ++i) {
        const v4 ci = tf4(tf, b, i);
        const real_t ni = gauss(density, *at3(tf, b, i, 4), *at3(tf, b, i, 5));
        acc.x += ci.x * ni; acc.y += ci.y * ni; acc.z += ci.z * ni; acc.w += ci.w * ni;
      }
      return acc;
    }
  }
}

/* TF adjoint; returns adj_density and scatters TF gradients when requested */
static real_t tf_adjoint(const OracleInputs* in, int b, real_t density, v4 adj, OracleAdjointOutputs* out) {
  const OracleTensor* tf = &in->tf;
  OracleTensor* g = &out->adj_tf;
  const int has_tf = out->has_tf;
  const int R = (int)tf->sizes[1];
  switch (in->tf_mode) {
    case 0: { /* :76-104 */
      const real_t dc = clampr(density, 0, 1);
      const real_t sa = *at3(tf, b, 0, 0), sc = *at3(tf, b, 0, 1);
      const real_t adj_dc = (adj.x * sc + adj.y * sc + adj.z * sc) + adj.w * sa;
      if (has_tf) {
        const real_t adj_sc = adj.x * dc + adj.y * dc + adj.z * dc;
        const real_t adj_sa = adj.w * dc;
        atomic_add(at3(g, b, 0, 0), adj_sa);
        atomic_add(at3(g, b, 0, 1), adj_sc);
      }
      return (density > 0 && density < 1) ? adj_dc : 0;
    }
    case 1: { /* :174-220 */
      const real_t d = density * R - (real_t)0.5;
      const int di = (int)floorf((float)d);
      const real_t df = d - di;
      const int i0 = clampi(di, 0, R - 1), i1 = clampi(di + 1, 0, R - 1);
      const v4 a = tf4(tf, b, i0), c = tf4(tf, b, i1);
      const real_t adj_df = dot4(adj, mk4(c.x - a.x, c.y - a.y, c.z - a.z, c.w - a.w));
      if (has_tf) {
        const real_t w0 = 1 - df;
        atomic_add(at3(g, b, i0, 0), adj.x * w0);
        atomic_add(at3(g, b, i0, 1), adj.y * w0);
        atomic_add(at3(g, b, i0, 2), adj.z * w0);
        atomic_add(at3(g, b, i0, 3), adj.w * w0);
        atomic_add(at3(g, b, i1, 0), adj.x * df);
        atomic_add(at3(g, b, i1, 1), adj.y * df);
        atomic_add(at3(g, b, i1, 2), adj.z * df);
        atomic_add(at3(g, b, i1, 3), adj.w * df);
      }
      /* passes adj_df * R even where the texel index was clamped (:219) */
      return adj_df * R;
    }
    case 2: { /* :316-400; the density gradient passes through the clamp (:350-351) */
      const int i = linear_interval(tf, b, R, density);
      const v4 a = tf4(tf, b, i), c = tf4(tf, b, i + 1);
      const real_t p0 = *at3(tf, b, i, 4), p1 = *at3(tf, b, i + 1, 4);
      const real_t d2 = clampr(density, p0, p1);
      const real_t fr = (d2 - p0) / (p1 - p0);
      const real_t adj_fr = dot4(adj, mk4(c.x - a.x, c.y - a.y, c.z - a.z, c.w - a.w));
      const real_t den = (p1 - p0) * (p1 - p0);
      const real_t adj_p0 = adj_fr * (d2 - p1) / den;
      const real_t adj_p1 = adj_fr * (p0 - d2) / den;
      const real_t adj_d2 = adj_fr / (p1 - p0);
      if (has_tf) {
        const real_t w0 = 1 - fr;
        atomic_add(at3(g, b, i, 0), adj.x * w0);
        atomic_add(at3(g, b, i, 1), adj.y * w0);
        atomic_add(at3(g, b, i, 2), adj.z * w0);
        atomic_add(at3(g, b, i, 3), adj.w * w0);
        atomic_add(at3(g, b, i, 4), adj_p0);
        atomic_add(at3(g, b, i + 1, 0), adj.x * fr);
        atomic_add(at3(g, b, i + 1, 1), adj.y * fr);
        atomic_add(at3(g, b, i + 1, 2), adj.z * fr);
        atomic_add(at3(g, b, i + 1, 3), adj.w * fr);
        atomic_add(at3(g, b, i + 1, 4), adj_p1);
      }
      return adj_d2;
    }
    default: { /* :563-614 */
      real_t adj_density = 0;
      for (int i = 0; i < R; ++i) {
        const v4 ci = tf4(tf, b, i);
        const real_t mu = *at3(tf, b, i, 4), sigma = *at3(tf, b, i, 5);
        const real_t s2 = sigma * sigma;
        const real_t ni = gauss(density, mu, sigma);
        const real_t f1 = (mu - density) / s2 * ni;
        adj_density += dot4(adj, mk4(ci.x * f1, ci.y * f1, ci.z * f1, ci.w * f1));
        if (has_tf) {
          const real_t nf1 = -f1;
          const real_t adj_mu = dot4(adj, mk4(ci.x * nf1, ci.y * nf1, ci.z * nf1, ci.w * nf1));
          /* the reference rounds this factor to float even in FP64 builds (:591) */
          const float f2 = (float)(f1 * (mu - density) / sigma);
          const real_t adj_sigma = dot4(adj, mk4(ci.x * f2, ci.y * f2, ci.z * f2, ci.w * f2));
          atomic_add(at3(g, b, i, 0), adj.x * ni);
          atomic_add(at3(g, b, i, 1), adj.y * ni);
          atomic_add(at3(g, b, i, 2), adj.z * ni);
          atomic_add(at3(g, b, i, 3), adj.w * ni);
          atomic_add(at3(g, b, i, 4), adj_mu);
          atomic_add(at3(g, b, i, 5), adj_sigma);
        }
      }
      return adj_density;
    }
  }
}

/* ---- blending (renderer/renderer_blending.cuh) ---- */
static inline real_t blend_alpha(int mode, real_t absorption, real_t step) {
  if (mode == 0) return 1 - R_EXP(-absorption * step);  /* Beer-Lambert (:54-61) */
  return rmin(1, absorption * step);                     /* alpha (:118-125) */
}

static inline v4 blend(int mode, v4 acc, v4 cur, real_t step) {
  const real_t a = blend_alpha(mode, cur.w, step);
  const real_t t = 1 - acc.w;
  return mk4(acc.x + t * cur.x * a, acc.y + t * cur.y * a, acc.z + t * cur.z * a, acc.w + t * a);
}

/* Adjoint of one blend step that inverts the blend to recover the accumulator
 * before the step (:63-98, :127-164).  adj_acc is updated in place; the step
 * size adjoint is ASSIGNED, reproducing the reference's behaviour. */
static v4 blend_adjoint(int mode, v4 acc_out, v4 cur, real_t step, v4* adj_acc, v4* adj_cur, real_t* adj_step) {
  const v4 ao = *adj_acc;
  real_t a;
  if (mode == 0) a = 1 - R_EXP(-cur.w * step);
  else a = rmin((real_t)(1 - (real_t)1e-5), cur.w * step);
  const real_t alpha_in = (a - acc_out.w) / (a - 1);
  const real_t t = 1 - alpha_in;
  v4 prev = mk4(acc_out.x - t * cur.x * a, acc_out.y - t * cur.y * a, acc_out.z - t * cur.z * a, alpha_in);
  real_t adj_alpha = ao.w * (1 - alpha_in);
  real_t adj_in_alpha = ao.w * (1 - a);
  adj_alpha += ao.x * (cur.x - cur.x * alpha_in) + ao.y * (cur.y - cur.y * alpha_in) +
               ao.z * (cur.z - cur.z * alpha_in);
  adj_in_alpha += ao.x * (-cur.x * a) + ao.y * (-cur.y * a) + ao.z * (-cur.z * a);
  const real_t wc = a * (1 - alpha_in);
  real_t adj_w;
  if (mode == 0) {
    adj_w = adj_alpha * step * R_EXP(-cur.w * step);
    *adj_step = adj_alpha * cur.w * R_EXP(-cur.w * step);
  } else {
    const int lin = cur.w * step < 1;
    *adj_step = lin ? adj_alpha * cur.w : 0;
    adj_w = lin ? adj_alpha * step : 0;
  }
  *adj_cur = mk4(ao.x * wc, ao.y * wc, ao.z * wc, adj_w);
  *adj_acc = mk4(ao.x, ao.y, ao.z, adj_in_alpha);
  return prev;
}

/* ---- per-ray setup shared by forward and adjoint ---- */
typedef struct {
  v3 start, dir, bmin, voxel;
  real_t step, tmin, tmax;
} RaySetup;

static void ray_setup(const OracleInputs* in, int x, int y, int b, RaySetup* r) {
  const OracleTensor* vol = &in->volume;
  r->bmin = mk3(*at2(&in->box_min, b, 0), *at2(&in->box_min, b, 1), *at2(&in->box_min, b, 2));
  const v3 bsize = mk3(*at2(&in->box_size, b, 0), *at2(&in->box_size, b, 1), *at2(&in->box_size, b, 2));
  r->voxel = mk3(bsize.x / (real_t)(vol->sizes[1] - 1), bsize.y / (real_t)(vol->sizes[2] - 1),
                 bsize.z / (real_t)(vol->sizes[3] - 1));
  compute_ray(in, x, y, b, &r->start, &r->dir);
  r->step = *at3(&in->step_size, b, y, x);
  ray_box(r->start, r->dir, r->bmin, bsize, &r->tmin, &r->tmax);
  r->tmin = rmax(r->tmin, 0);
}

static inline v3 volume_pos(const RaySetup* r, real_t t) {
  const v3 w = mk3(r->start.x + t * r->dir.x, r->start.y + t * r->dir.y, r->start.z + t * r->dir.z);
  return mk3((w.x - r->bmin.x) / r->voxel.x, (w.y - r->bmin.y) / r->voxel.y, (w.z - r->bmin.z) / r->voxel.z);
}

/* adjoint of volumePos = (start + t*dir - boxMin) / voxelSize at t = tmin + k*step,
 * tmin held fixed (:407-412): accumulates into the ray start, direction and step */
static inline void ray_step_adjoint(const RaySetup* r, real_t t, int k, v3 adj_vp, v3* adj_start, v3* adj_dir,
                                    real_t* adj_step) {
  const v3 adj_w = mk3(adj_vp.x / r->voxel.x, adj_vp.y / r->voxel.y, adj_vp.z / r->voxel.z);
  adj_start->x += adj_w.x; adj_start->y += adj_w.y; adj_start->z += adj_w.z;
  adj_dir->x += adj_w.x * t; adj_dir->y += adj_w.y * t; adj_dir->z += adj_w.z * t;
  const real_t adj_t = dot3(adj_w, r->dir);
  *adj_step += adj_t * k;
}

static int check_modes(const OracleInputs* in) {
  /* pre-shaded: filter 3 together with TF 5 (renderer/renderer.cpp:72-80) */
  const int preshaded = in->filter_mode == 3;
  if (preshaded != (in->tf_mode == 5)) return 2;
  if (!preshaded && (in->filter_mode < 0 || in->filter_mode > 1)) return 2;
  if (in->camera_mode < 0 || in->camera_mode > 2) return 2;
  if (!preshaded && (in->tf_mode < 0 || in->tf_mode > 3)) return 2;
  if (in->blend_mode < 0 || in->blend_mode > 1) return 2;
  if (preshaded && in->volume.sizes[0] != 4) return 2;
  return 0;
}

/* ---- pre-shaded volumes (renderer/renderer_interpolation.cuh:393-579,
 *      renderer/renderer_tf.cuh:818-854): the volume is 4 X Y Z, the colour
 *      and absorption channels in its first dimension, shared by all batch
 *      entries; each channel is interpolated trilinearly and the TF passes
 *      the result through. ---- */
static int g_exact_preshaded = 0;
/* 0 (default): the reference's position adjoint, whose z term is summed
 * with the y weights' selector (renderer/renderer_interpolation.cuh:543-548);
 * 1: the exact trilinear z derivative. */
void oracle_set_exact_preshaded(int exact) { g_exact_preshaded = exact; }

typedef struct {
  const OracleTensor* vol;
  OracleTensor* adj;
  int has_adj;
  int X, Y, Z;
  int li[3];
  real_t dens[4][8];
  real_t acc[4][8];
  real_t fpos[3];
} RgbaSampler;

static void rgba_corners(const RgbaSampler* s, const int* ip, real_t d[4][8]) {
  const int lx = clampi(ip[0], 0, s->X - 1), hx = clampi(ip[0] + 1, 0, s->X - 1);
  const int ly = clampi(ip[1], 0, s->Y - 1), hy = clampi(ip[1] + 1, 0, s->Y - 1);
  const int lz = clampi(ip[2], 0, s->Z - 1), hz = clampi(ip[2] + 1, 0, s->Z - 1);
  for (int c = 0; c < 4; ++c) {
    d[c][0] = *at4(s->vol, c, lx, ly, lz); d[c][1] = *at4(s->vol, c, lx, ly, hz);
    d[c][2] = *at4(s->vol, c, lx, hy, lz); d[c][3] = *at4(s->vol, c, lx, hy, hz);
    d[c][4] = *at4(s->vol, c, hx, ly, lz); d[c][5] = *at4(s->vol, c, hx, ly, hz);
    d[c][6] = *at4(s->vol, c, hx, hy, lz); d[c][7] = *at4(s->vol, c, hx, hy, hz);
  }
}

static v4 rgba_forward(const RgbaSampler* s, v3 p) {
  int ip[3] = {(int)p.x, (int)p.y, (int)p.z};
  real_t d[4][8], f[3] = {p.x - (real_t)ip[0], p.y - (real_t)ip[1], p.z - (real_t)ip[2]};
  rgba_corners(s, ip, d);
  return mk4(trilerp(d[0], f), trilerp(d[1], f), trilerp(d[2], f), trilerp(d[3], f));
}

static void rgba_flush(RgbaSampler* s) {
  if (!s->has_adj || s->li[0] < 0) return;
  const int lx = clampi(s->li[0], 0, s->X - 1), hx = clampi(s->li[0] + 1, 0, s->X - 1);
  const int ly = clampi(s->li[1], 0, s->Y - 1), hy = clampi(s->li[1] + 1, 0, s->Y - 1);
  const int lz = clampi(s->li[2], 0, s->Z - 1), hz = clampi(s->li[2] + 1, 0, s->Z - 1);
  for (int c = 0; c < 4; ++c) {
    atomic_add(at4(s->adj, c, lx, ly, lz), s->acc[c][0]);
    atomic_add(at4(s->adj, c, lx, ly, hz), s->acc[c][1]);
    atomic_add(at4(s->adj, c, lx, hy, lz), s->acc[c][2]);
    atomic_add(at4(s->adj, c, lx, hy, hz), s->acc[c][3]);
    atomic_add(at4(s->adj, c, hx, ly, lz), s->acc[c][4]);
    atomic_add(at4(s->adj, c, hx, ly, hz), s->acc[c][5]);
    atomic_add(at4(s->adj, c, hx, hy, lz), s->acc[c][6]);
    atomic_add(at4(s->adj, c, hx, hy, hz), s->acc[c][7]);
    for (int i = 0; i < 8; ++i) s->acc[c][i] = 0;
  }
}

static v4 rgba_adjoint_fetch(RgbaSampler* s, v3 p) {
  int ip[3] = {(int)p.x, (int)p.y, (int)p.z};
  if (ip[0] != s->li[0] || ip[1] != s->li[1] || ip[2] != s->li[2]) {
    rgba_flush(s);
    s->li[0] = ip[0]; s->li[1] = ip[1]; s->li[2] = ip[2];
    rgba_corners(s, ip, s->dens);
  }
  s->fpos[0] = p.x - (real_t)ip[0];
  s->fpos[1] = p.y - (real_t)ip[1];
  s->fpos[2] = p.z - (real_t)ip[2];
  return mk4(trilerp(s->dens[0], s->fpos), trilerp(s->dens[1], s->fpos), trilerp(s->dens[2], s->fpos),
             trilerp(s->dens[3], s->fpos));
}

/* adjoint of the four trilinear channels; returns d(colour)/d(volumePos) . adj */
static v3 rgba_adjoint(RgbaSampler* s, v4 adj) {
  const real_t c[3] = {s->fpos[0], s->fpos[1], s->fpos[2]};
  const real_t f[3] = {1 - c[0], 1 - c[1], 1 - c[2]};
  real_t adj_c[3] = {0, 0, 0}, adj_f[3] = {0, 0, 0};
  const real_t a[4] = {adj.x, adj.y, adj.z, adj.w};
  static const int order[8] = {0, 4, 2, 6, 1, 5, 3, 7};
  for (int ch = 0; ch < 4; ++ch)
    for (int k = 0; k < 8; ++k) {
      const int idx = order[k];
      const int hx = (idx >> 2) & 1, hy = (idx >> 1) & 1, hz = idx & 1;
      const real_t wx = hx ? c[0] : f[0], wy = hy ? c[1] : f[1], wz = hz ? c[2] : f[2];
      if (s->has_adj) s->acc[ch][idx] += a[ch] * (wx * wy * wz);
      (hx ? adj_c : adj_f)[0] += a[ch] * s->dens[ch][idx] * wy * wz;
      (hy ? adj_c : adj_f)[1] += a[ch] * s->dens[ch][idx] * wx * wz;
      (g_exact_preshaded ? (hz ? adj_c : adj_f) : (hy ? adj_c : adj_f))[2] += a[ch] * s->dens[ch][idx] * wx * wy;
    }
  return mk3(adj_c[0] - adj_f[0], adj_c[1] - adj_f[1], adj_c[2] - adj_f[2]);
}

int oracle_real_size(void) { return (int)sizeof(real_t); }

/* Threads of the parallel loops started from the calling thread from now on
 * (the OpenMP runtime is shared by every library of the process, the
 * reference's templates included); returns the previous number.  One thread
 * makes the atomic sums of the adjoint deterministic. */
int oracle_set_threads(int n) {
#ifdef _OPENMP
  const int prev = omp_get_max_threads();
  if (n > 0) omp_set_num_threads(n);
  return prev;
#else
  (void)n;
  return 1;
#endif
}

/* ---- forward march (renderer/renderer_kernels.cuh:22-90) ---- */
int oracle_forward(const OracleInputs* in, OracleTensor* color, OracleTensor* termination) {
  if (check_modes(in)) return 2;
  const int W = in->width, H = in->height, B = in->batch;
  const int64_t count = (int64_t)W * H * B;
  const real_t early_out = (real_t)in->blending_early_out;
#pragma omp parallel for schedule(guided)
  for (int64_t i = 0; i < count; ++i) {
    const int b = (int)(i / ((int64_t)W * H));
    const int y = (int)((i - (int64_t)b * W * H) / W);
    const int x = (int)(i - (int64_t)W * (y + (int64_t)H * b));
    RaySetup r;
    ray_setup(in, x, y, b, &r);
    Sampler s = {b, (int)in->volume.sizes[1], (int)in->volume.sizes[2], (int)in->volume.sizes[3], &in->volume};
    RgbaSampler rs = {&in->volume, NULL, 0, s.X, s.Y, s.Z};
    v4 acc = mk4(0, 0, 0, 0);
    int k;
    for (k = 0;; ++k) {
      const real_t t = r.tmin + k * r.step;
      if (t > r.tmax) break;
      if (acc.w > early_out) break;
      v4 cur;
      if (in->filter_mode == 3) {
        cur = rgba_forward(&rs, volume_pos(&r, t));
      } else {
        const real_t density = sample_forward(&s, in->filter_mode, volume_pos(&r, t));
        cur = tf_eval(in, b, density);
      }
      acc = blend(in->blend_mode, acc, cur, r.step);
    }
    *at4(color, b, y, x, 0) = acc.x;
    *at4(color, b, y, x, 1) = acc.y;
    *at4(color, b, y, x, 2) = acc.z;
    *at4(color, b, y, x, 3) = acc.w;
    *iat3(termination, b, y, x) = k;
  }
  return 0;
}

/* ---- adjoint march (renderer/renderer_kernels.cuh:315-444) ---- */
int oracle_adjoint(const OracleInputs* in, const OracleTensor* color, const OracleTensor* termination,
                   const OracleTensor* adj_color, OracleAdjointOutputs* out) {
  if (check_modes(in)) return 2;
  if (!out->has_volume && !out->has_stepsize && !out->has_camera && !out->has_tf) return 3;
  const int W = in->width, H = in->height, B = in->batch;
  const int64_t count = (int64_t)W * H * B;
#pragma omp parallel for schedule(guided)
  for (int64_t i = 0; i < count; ++i) {
    const int b = (int)(i / ((int64_t)W * H));
    const int y = (int)((i - (int64_t)b * W * H) / W);
    const int x = (int)(i - (int64_t)W * (y + (int64_t)H * b));
    RaySetup r;
    ray_setup(in, x, y, b, &r);
    v4 acc = mk4(*at4(color, b, y, x, 0), *at4(color, b, y, x, 1), *at4(color, b, y, x, 2), *at4(color, b, y, x, 3));
    int k = *iat3(termination, b, y, x);
    v4 adj_acc = mk4(*at4(adj_color, b, y, x, 0), *at4(adj_color, b, y, x, 1), *at4(adj_color, b, y, x, 2),
                     *at4(adj_color, b, y, x, 3));
    real_t adj_step = 0;
    v3 adj_start = mk3(0, 0, 0), adj_dir = mk3(0, 0, 0);
    Sampler s = {b, (int)in->volume.sizes[1], (int)in->volume.sizes[2], (int)in->volume.sizes[3], &in->volume};
    s.adj = &out->adj_volume;
    s.has_adj = out->has_volume;
    s.li[0] = s.li[1] = s.li[2] = -1;
    for (int q = 0; q < 8; ++q) s.acc[q] = s.dens[q] = 0;
    s.nearest_val = s.nearest_acc = 0;
    RgbaSampler rs;
    rs.vol = &in->volume;
    rs.adj = &out->adj_volume;
    rs.has_adj = out->has_volume;
    rs.X = s.X; rs.Y = s.Y; rs.Z = s.Z;
    rs.li[0] = rs.li[1] = rs.li[2] = -1;
    for (int c = 0; c < 4; ++c)
      for (int q = 0; q < 8; ++q) rs.acc[c][q] = rs.dens[c][q] = 0;
    /* the last blended sample has index terminationIndex-1 (:374-376) */
    for (--k; k >= 0; --k) {
      const real_t t = r.tmin + k * r.step;
      v3 adj_vp;
      v4 adj_cur;
      if (in->filter_mode == 3) {
        /* the TF passes the colour through, and its adjoint the colour adjoint */
        const v4 cur = rgba_adjoint_fetch(&rs, volume_pos(&r, t));
        acc = blend_adjoint(in->blend_mode, acc, cur, r.step, &adj_acc, &adj_cur, &adj_step);
        adj_vp = rgba_adjoint(&rs, adj_cur);
      } else {
        const real_t density = sample_adjoint_fetch(&s, in->filter_mode, volume_pos(&r, t));
        const v4 cur = tf_eval(in, b, density);
        acc = blend_adjoint(in->blend_mode, acc, cur, r.step, &adj_acc, &adj_cur, &adj_step);
        const real_t adj_density = tf_adjoint(in, b, density, adj_cur, out);
        adj_vp = sample_adjoint(&s, in->filter_mode, adj_density);
      }
      ray_step_adjoint(&r, t, k, adj_vp, &adj_start, &adj_dir, &adj_step);
    }
    if (in->filter_mode == 3) rgba_flush(&rs);
    else sampler_flush(&s, in->filter_mode);
    if (out->has_stepsize) {
      real_t* p = at3(&out->adj_stepsize, b, y, x);
      if (out->stepsize_broadcast) atomic_add(p, adj_step);
      else *p = adj_step;
    }
    if (out->has_camera) {
      real_t* ps[3] = {at4(&out->adj_ray_start, b, y, x, 0), at4(&out->adj_ray_start, b, y, x, 1),
                       at4(&out->adj_ray_start, b, y, x, 2)};
      real_t* pd[3] = {at4(&out->adj_ray_dir, b, y, x, 0), at4(&out->adj_ray_dir, b, y, x, 1),
                       at4(&out->adj_ray_dir, b, y, x, 2)};
      const real_t vs[3] = {adj_start.x, adj_start.y, adj_start.z};
      const real_t vd[3] = {adj_dir.x, adj_dir.y, adj_dir.z};
      for (int c = 0; c < 3; ++c) {
        if (out->camera_broadcast) { atomic_add(ps[c], vs[c]); atomic_add(pd[c], vd[c]); }
        else { *ps[c] = vs[c]; *pd[c] = vd[c]; }
      }
    }
  }
  return 0;
}

/* ---- forward-mode differentiation (renderer/renderer_kernels.cuh:131-240) ----
 * Every traced quantity carries, next to its value, its D partial derivatives
 * with respect to the variables the settings select: the step size, the
 * components of the ray start and direction (after ray generation), and TF
 * entries (each with its own index, renderer/renderer_settings.cuh:189-206).
 * The values are computed by the same functions as oracle_forward, so colour
 * and termination index are identical; the derivatives follow the chain rule
 * through the position, the density (trilinear gradient; nearest sampling
 * has none), the TF and the blend.  The entry and exit distances are not
 * traced (:201-207).  The reference's dual-number type (cudAD) is not part of
 * the reference sources, so this restates the derivatives directly. */

static inline real_t* at5(const OracleTensor* t, int64_t i0, int64_t i1, int64_t i2, int64_t i3, int64_t i4) {
  return (real_t*)t->data + i0 * bstride(t, 0) + i1 * bstride(t, 1) + i2 * bstride(t, 2) + i3 * bstride(t, 3) +
         i4 * bstride(t, 4);
}

/* derivative index of TF entry (r, c), or -1 */
static inline int tf_index(const OracleForwardSettings* fs, int b, int r, int c) {
  if (!fs->has_tf) return -1;
  const int i = *iat3(&fs->d_tf, b, r, c);
  return (i >= 0 && i < fs->D) ? i : -1;
}

static inline int var_index(int i, int D) { return (i >= 0 && i < D) ? i : -1; }

/* Derivatives of the TF colour: dc[ch * D + j] = d c_ch / d var_j, given the
 * density's derivatives dden (renderer/renderer_tf.cuh:122-150, :256-290,
 * :437-486, :522-560).  Clamps select an operand together with its
 * derivatives: the identity TF's density clamp passes the derivative only
 * strictly inside (0, 1), like its adjoint; the linear TF's density clamp to
 * [p0, p1] takes the derivative of the bound it clamps to. */
static void tf_dual(const OracleInputs* in, const OracleForwardSettings* fs, int b, real_t density,
                    const real_t* dden, real_t* dc) {
  const OracleTensor* tf = &in->tf;
  const int R = (int)tf->sizes[1];
  const int D = fs->D;
  for (int j = 0; j < 4 * D; ++j) dc[j] = 0;
  switch (in->tf_mode) {
    case 0: {
      const real_t dcl = clampr(density, 0, 1);
      const int inside = density > 0 && density < 1;
      const real_t sa = *at3(tf, b, 0, 0), sc = *at3(tf, b, 0, 1);
      if (inside)
        for (int j = 0; j < D; ++j) {
          dc[0 * D + j] = dden[j] * sc;
          dc[1 * D + j] = dden[j] * sc;
          dc[2 * D + j] = dden[j] * sc;
          dc[3 * D + j] = dden[j] * sa;
        }
      const int isa = tf_index(fs, b, 0, 0), isc = tf_index(fs, b, 0, 1);
      if (isa >= 0) dc[3 * D + isa] += dcl;
      if (isc >= 0) { dc[0 * D + isc] += dcl; dc[1 * D + isc] += dcl; dc[2 * D + isc] += dcl; }
      break;
    }
    case 1: {
      const real_t d = density * R - (real_t)0.5;
      const int di = (int)floorf((float)d);
      const real_t df = d - di;
      const int i0 = clampi(di, 0, R - 1), i1 = clampi(di + 1, 0, R - 1);
      const v4 a = tf4(tf, b, i0), c = tf4(tf, b, i1);
      const real_t dv[4] = {c.x - a.x, c.y - a.y, c.z - a.z, c.w - a.w};
      for (int ch = 0; ch < 4; ++ch)
        for (int j = 0; j < D; ++j) dc[ch * D + j] = dv[ch] * (R * dden[j]);
      for (int ch = 0; ch < 4; ++ch) {
        const int k0 = tf_index(fs, b, i0, ch), k1 = tf_index(fs, b, i1, ch);
        if (k0 >= 0) dc[ch * D + k0] += 1 - df;
        if (k1 >= 0) dc[ch * D + k1] += df;
      }
      break;
    }
    case 2: {
      const int i = linear_interval(tf, b, R, density);
      const v4 a = tf4(tf, b, i), c = tf4(tf, b, i + 1);
      const real_t p0 = *at3(tf, b, i, 4), p1 = *at3(tf, b, i + 1, 4);
      const int lo = density < p0, hi = !lo && density > p1;
      const real_t d2 = lo ? p0 : (hi ? p1 : density);
      const real_t den = p1 - p0;
      const real_t fr = (d2 - p0) / den;
      const real_t dv[4] = {c.x - a.x, c.y - a.y, c.z - a.z, c.w - a.w};
      const int ip0 = tf_index(fs, b, i, 4), ip1 = tf_index(fs, b, i + 1, 4);
      for (int j = 0; j < D; ++j) {
        const real_t dp0 = j == ip0 ? 1 : 0, dp1 = j == ip1 ? 1 : 0;
        const real_t dd2 = lo ? dp0 : (hi ? dp1 : dden[j]);
        const real_t dfr = ((dd2 - dp0) * den - (d2 - p0) * (dp1 - dp0)) / (den * den);
        for (int ch = 0; ch < 4; ++ch) dc[ch * D + j] = dv[ch] * dfr;
      }
      for (int ch = 0; ch < 4; ++ch) {
        const int k0 = tf_index(fs, b, i, ch), k1 = tf_index(fs, b, i + 1, ch);
        if (k0 >= 0) dc[ch * D + k0] += 1 - fr;
        if (k1 >= 0) dc[ch * D + k1] += fr;
      }
      break;
    }
    default: {
      for (int i = 0; i < R; ++i) {
        const v4 ci = tf4(tf, b, i);
        const real_t cv[4] = {ci.x, ci.y, ci.z, ci.w};
        const real_t mu = *at3(tf, b, i, 4), sigma = *at3(tf, b, i, 5);
        const real_t ni = gauss(density, mu, sigma);
        const real_t s2 = sigma * sigma;
        const int imu = tf_index(fs, b, i, 4), isg = tf_index(fs, b, i, 5);
        for (int j = 0; j < D; ++j) {
          const real_t dmu = j == imu ? 1 : 0, dsg = j == isg ? 1 : 0;
          const real_t dn = ni * (-(density - mu) * (dden[j] - dmu) / s2 +
                                  (density - mu) * (density - mu) * dsg / (s2 * sigma));
          for (int ch = 0; ch < 4; ++ch) dc[ch * D + j] += cv[ch] * dn;
        }
        for (int ch = 0; ch < 4; ++ch) {
          const int k = tf_index(fs, b, i, ch);
          if (k >= 0) dc[ch * D + k] += ni;
        }
      }
      break;
    }
  }
}

/* trilinear density and its gradient with respect to the volume position */
static real_t trilerp_grad(const real_t* d, const real_t* f, v3* g) {
  const real_t ay0 = lerp1(d[0], d[4], f[0]), ay1 = lerp1(d[2], d[6], f[0]);
  const real_t by0 = lerp1(d[1], d[5], f[0]), by1 = lerp1(d[3], d[7], f[0]);
  g->x = lerp1(lerp1(d[4] - d[0], d[6] - d[2], f[1]), lerp1(d[5] - d[1], d[7] - d[3], f[1]), f[2]);
  g->y = lerp1(ay1 - ay0, by1 - by0, f[2]);
  g->z = lerp1(by0, by1, f[1]) - lerp1(ay0, ay1, f[1]);
  return lerp1(lerp1(ay0, ay1, f[1]), lerp1(by0, by1, f[1]), f[2]);
}

int oracle_forward_gradients(const OracleInputs* in, const OracleForwardSettings* fs, OracleTensor* color,
                             OracleTensor* termination, OracleTensor* grads) {
  if (check_modes(in) || in->filter_mode == 3) return 2;
  const int D = fs->D;
  if (D <= 0) return 3;
  const int W = in->width, H = in->height, B = in->batch;
  const int64_t count = (int64_t)W * H * B;
  const real_t early_out = (real_t)in->blending_early_out;
  const int istep = var_index(fs->d_stepsize, D);
  int istart[3], idir[3];
  for (int c = 0; c < 3; ++c) {
    istart[c] = var_index(fs->d_ray_start[c], D);
    idir[c] = var_index(fs->d_ray_dir[c], D);
  }
  int failed = 0;
#pragma omp parallel for schedule(guided)
  for (int64_t i = 0; i < count; ++i) {
    const int b = (int)(i / ((int64_t)W * H));
    const int y = (int)((i - (int64_t)b * W * H) / W);
    const int x = (int)(i - (int64_t)W * (y + (int64_t)H * b));
    /* derivative arrays of one ray: start, dir, step, volume position,
     * density, TF colour, alpha, accumulator */
    real_t* buf = (real_t*)calloc((size_t)D * 21, sizeof(real_t));
    if (!buf) {
#pragma omp atomic write
      failed = 1;
      continue;
    }
    real_t *dstart = buf, *ddir = buf + 3 * D, *dstep = buf + 6 * D, *dvp = buf + 7 * D, *dden = buf + 10 * D;
    real_t *dc = buf + 11 * D, *dalpha = buf + 15 * D, *dacc = buf + 16 * D;
    RaySetup r;
    ray_setup(in, x, y, b, &r);
    for (int c = 0; c < 3; ++c) {
      if (istart[c] >= 0) dstart[c * D + istart[c]] = 1;
      if (idir[c] >= 0) ddir[c * D + idir[c]] = 1;
    }
    if (istep >= 0) dstep[istep] = 1;
    const real_t dirv[3] = {r.dir.x, r.dir.y, r.dir.z};
    const real_t vox3[3] = {r.voxel.x, r.voxel.y, r.voxel.z};
    Sampler s = {b, (int)in->volume.sizes[1], (int)in->volume.sizes[2], (int)in->volume.sizes[3], &in->volume};
    v4 acc = mk4(0, 0, 0, 0);
    int k;
    for (k = 0;; ++k) {
      const real_t t = r.tmin + k * r.step;
      if (t > r.tmax) break;
      if (acc.w > early_out) break;
      const v3 p = volume_pos(&r, t);
      /* volumePos = (start + t dir - boxMin) / voxelSize, t = tmin + k step */
      for (int c = 0; c < 3; ++c)
        for (int j = 0; j < D; ++j)
          dvp[c * D + j] = (dstart[c * D + j] + k * dstep[j] * dirv[c] + t * ddir[c * D + j]) / vox3[c];
      real_t density;
      if (in->filter_mode == 0) {
        density = sample_forward(&s, 0, p);
        for (int j = 0; j < D; ++j) dden[j] = 0;
      } else {
        int ip[3] = {(int)p.x, (int)p.y, (int)p.z};
        real_t d8[8], f[3] = {p.x - (real_t)ip[0], p.y - (real_t)ip[1], p.z - (real_t)ip[2]};
        cell_corners(&s, ip, d8);
        v3 g;
        trilerp_grad(d8, f, &g);
        density = trilerp(d8, f);
        for (int j = 0; j < D; ++j) dden[j] = g.x * dvp[j] + g.y * dvp[D + j] + g.z * dvp[2 * D + j];
      }
      const v4 cur = tf_eval(in, b, density);
      tf_dual(in, fs, b, density, dden, dc);
      const real_t a = blend_alpha(in->blend_mode, cur.w, r.step);
      if (in->blend_mode == 0) {
        const real_t e = R_EXP(-cur.w * r.step);
        for (int j = 0; j < D; ++j) dalpha[j] = e * (dc[3 * D + j] * r.step + cur.w * dstep[j]);
      } else {
        const int lin = cur.w * r.step < 1;
        for (int j = 0; j < D; ++j) dalpha[j] = lin ? dc[3 * D + j] * r.step + cur.w * dstep[j] : 0;
      }
      /* colorOut = acc + (1 - acc.w) c alpha, alphaOut = acc.w + (1 - acc.w) alpha
       * (renderer/renderer_blending.cuh:40-52) */
      const real_t T = 1 - acc.w;
      const real_t cv[3] = {cur.x, cur.y, cur.z};
      for (int j = 0; j < D; ++j) {
        const real_t dT = -dacc[3 * D + j];
        for (int c = 0; c < 3; ++c)
          dacc[c * D + j] += dT * cv[c] * a + T * dc[c * D + j] * a + T * cv[c] * dalpha[j];
        dacc[3 * D + j] += dT * a + T * dalpha[j];
      }
      acc = blend(in->blend_mode, acc, cur, r.step);
    }
    *at4(color, b, y, x, 0) = acc.x;
    *at4(color, b, y, x, 1) = acc.y;
    *at4(color, b, y, x, 2) = acc.z;
    *at4(color, b, y, x, 3) = acc.w;
    *iat3(termination, b, y, x) = k;
    for (int j = 0; j < D; ++j)
      for (int c = 0; c < 4; ++c) *at5(grads, b, y, x, j, c) = dacc[c * D + j];
    free(buf);
  }
  return failed ? 4 : 0;
}

/* renderer/renderer_kernels.cuh:505-560: per pixel, each enabled variable's
 * gradient is dot(adj_color, d color / d variable); step size and camera
 * gradients are per pixel (accumulated where their output broadcasts), TF
 * gradients accumulate over the pixels. */
int oracle_forward_variables_to_gradients(const OracleTensor* fwd, const OracleTensor* adj_color,
                                          const OracleForwardSettings* fs, OracleAdjointOutputs* out) {
  const int B = (int)fwd->sizes[0], H = (int)fwd->sizes[1], W = (int)fwd->sizes[2], D = (int)fwd->sizes[3];
  if (D != fs->D) return 3;
  const int64_t count = (int64_t)W * H * B;
  const int istep = var_index(fs->d_stepsize, D);
  const int R = fs->has_tf ? (int)fs->d_tf.sizes[1] : 0, C = fs->has_tf ? (int)fs->d_tf.sizes[2] : 0;
#pragma omp parallel for schedule(guided)
  for (int64_t i = 0; i < count; ++i) {
    const int b = (int)(i / ((int64_t)W * H));
    const int y = (int)((i - (int64_t)b * W * H) / W);
    const int x = (int)(i - (int64_t)W * (y + (int64_t)H * b));
    const v4 g = mk4(*at4(adj_color, b, y, x, 0), *at4(adj_color, b, y, x, 1), *at4(adj_color, b, y, x, 2),
                     *at4(adj_color, b, y, x, 3));
#define FWD4(j) mk4(*at5(fwd, b, y, x, j, 0), *at5(fwd, b, y, x, j, 1), *at5(fwd, b, y, x, j, 2), *at5(fwd, b, y, x, j, 3))
    if (out->has_stepsize && istep >= 0) {
      real_t* p = at3(&out->adj_stepsize, b, y, x);
      const real_t v = dot4(g, FWD4(istep));
      if (out->stepsize_broadcast) atomic_add(p, v);
      else *p = v;
    }
    if (out->has_camera)
      for (int c = 0; c < 3; ++c) {
        const int is = var_index(fs->d_ray_start[c], D), id = var_index(fs->d_ray_dir[c], D);
        if (is >= 0) {
          real_t* p = at4(&out->adj_ray_start, b, y, x, c);
          const real_t v = dot4(g, FWD4(is));
          if (out->camera_broadcast) atomic_add(p, v);
          else *p = v;
        }
        if (id >= 0) {
          real_t* p = at4(&out->adj_ray_dir, b, y, x, c);
          const real_t v = dot4(g, FWD4(id));
          if (out->camera_broadcast) atomic_add(p, v);
          else *p = v;
        }
      }
    if (out->has_tf && fs->has_tf)
      for (int r = 0; r < R; ++r)
        for (int c = 0; c < C; ++c) {
          const int k = tf_index(fs, b, r, c);
          if (k >= 0) atomic_add(at3(&out->adj_tf, b, r, c), dot4(g, FWD4(k)));
        }
#undef FWD4
  }
  return 0;
}

/* ---- pre-shading (renderer/tf_utils_impl.cu:16-31, :120-140): a density
 * volume 1 X Y Z becomes the colour volume 4 X Y Z through the TF of batch
 * entry 0; the adjoint writes d loss / d density per voxel. ---- */
static void preshade_inputs(const OracleTensor* tf, int tf_mode, OracleInputs* in) {
  OracleInputs z = {0};
  *in = z;
  in->tf = *tf;
  in->tf_mode = tf_mode;
}

int oracle_preshade_volume(const OracleTensor* density, const OracleTensor* tf, int tf_mode, OracleTensor* color) {
  if (tf_mode < 0 || tf_mode > 3) return 2;
  OracleInputs in;
  preshade_inputs(tf, tf_mode, &in);
  const int X = (int)density->sizes[1], Y = (int)density->sizes[2], Z = (int)density->sizes[3];
#pragma omp parallel for schedule(static)
  for (int x = 0; x < X; ++x)
    for (int y = 0; y < Y; ++y)
      for (int z = 0; z < Z; ++z) {
        const v4 c = tf_eval(&in, 0, *at4(density, 0, x, y, z));
        *at4(color, 0, x, y, z) = c.x;
        *at4(color, 1, x, y, z) = c.y;
        *at4(color, 2, x, y, z) = c.z;
        *at4(color, 3, x, y, z) = c.w;
      }
  return 0;
}

int oracle_preshade_volume_adjoint(const OracleTensor* density, const OracleTensor* tf, int tf_mode,
                                   const OracleTensor* adj_color, OracleTensor* adj_density) {
  if (tf_mode < 0 || tf_mode > 3) return 2;
  OracleInputs in;
  preshade_inputs(tf, tf_mode, &in);
  OracleAdjointOutputs none;
  OracleAdjointOutputs z = {0};
  none = z;  /* no TF gradient (:126-129) */
  const int X = (int)density->sizes[1], Y = (int)density->sizes[2], Z = (int)density->sizes[3];
#pragma omp parallel for schedule(static)
  for (int x = 0; x < X; ++x)
    for (int y = 0; y < Y; ++y)
      for (int z = 0; z < Z; ++z) {
        const v4 a = mk4(*at4(adj_color, 0, x, y, z), *at4(adj_color, 1, x, y, z), *at4(adj_color, 2, x, y, z),
                         *at4(adj_color, 3, x, y, z));
        *at4(adj_density, 0, x, y, z) = tf_adjoint(&in, 0, *at4(density, 0, x, y, z), a, &none);
      }
  return 0;
}

/* ---- per-step components, exported for the per-component adjoint tests
 * (the reference's unittests/testAdjoint{Blending,TF,Interpolation,Camera}.cpp):
 * each runs the function the march above uses, on one step. */

int oracle_blend_step(int mode, const real_t* acc, const real_t* cur, real_t step, real_t* out) {
  const v4 r = blend(mode, mk4(acc[0], acc[1], acc[2], acc[3]), mk4(cur[0], cur[1], cur[2], cur[3]), step);
  out[0] = r.x; out[1] = r.y; out[2] = r.z; out[3] = r.w;
  return 0;
}

int oracle_blend_step_adjoint(int mode, const real_t* acc_out, const real_t* cur, real_t step, const real_t* adj_out,
                              real_t* acc_in, real_t* adj_acc_in, real_t* adj_cur, real_t* adj_step) {
  v4 aa = mk4(adj_out[0], adj_out[1], adj_out[2], adj_out[3]), ac;
  const v4 prev = blend_adjoint(mode, mk4(acc_out[0], acc_out[1], acc_out[2], acc_out[3]),
                                mk4(cur[0], cur[1], cur[2], cur[3]), step, &aa, &ac, adj_step);
  acc_in[0] = prev.x; acc_in[1] = prev.y; acc_in[2] = prev.z; acc_in[3] = prev.w;
  adj_acc_in[0] = aa.x; adj_acc_in[1] = aa.y; adj_acc_in[2] = aa.z; adj_acc_in[3] = aa.w;
  adj_cur[0] = ac.x; adj_cur[1] = ac.y; adj_cur[2] = ac.z; adj_cur[3] = ac.w;
  return 0;
}

int oracle_tf_step(const OracleTensor* tf, int tf_mode, real_t density, real_t* out) {
  if (tf_mode < 0 || tf_mode > 3) return 2;
  OracleInputs in;
  preshade_inputs(tf, tf_mode, &in);
  const v4 c = tf_eval(&in, 0, density);
  out[0] = c.x; out[1] = c.y; out[2] = c.z; out[3] = c.w;
  return 0;
}

int oracle_tf_step_adjoint(const OracleTensor* tf, int tf_mode, real_t density, const real_t* adj, OracleTensor* adj_tf,
                           real_t* adj_density) {
  if (tf_mode < 0 || tf_mode > 3) return 2;
  OracleInputs in;
  preshade_inputs(tf, tf_mode, &in);
  OracleAdjointOutputs out;
  memset(&out, 0, sizeof out);
  if (adj_tf && adj_tf->data) {
    out.has_tf = 1;
    out.adj_tf = *adj_tf;
  }
  *adj_density = tf_adjoint(&in, 0, density, mk4(adj[0], adj[1], adj[2], adj[3]), &out);
  return 0;
}

static void component_sampler(const OracleTensor* volume, OracleTensor* adj_volume, Sampler* s) {
  memset(s, 0, sizeof *s);
  s->X = (int)volume->sizes[1]; s->Y = (int)volume->sizes[2]; s->Z = (int)volume->sizes[3];
  s->vol = volume;
  s->adj = adj_volume;
  s->has_adj = adj_volume && adj_volume->data;
  s->li[0] = s->li[1] = s->li[2] = -1;
}

/* pos: volume (voxel) coordinates of batch entry 0 */
int oracle_sample_step(const OracleTensor* volume, int filter, const real_t* pos, real_t* density) {
  if (filter != 0 && filter != 1) return 2;
  Sampler s;
  component_sampler(volume, NULL, &s);
  *density = sample_forward(&s, filter, mk3(pos[0], pos[1], pos[2]));
  return 0;
}

int oracle_sample_step_adjoint(const OracleTensor* volume, int filter, const real_t* pos, real_t adj_density,
                               real_t* adj_pos, OracleTensor* adj_volume) {
  if (filter != 0 && filter != 1) return 2;
  Sampler s;
  component_sampler(volume, adj_volume, &s);
  (void)sample_adjoint_fetch(&s, filter, mk3(pos[0], pos[1], pos[2]));
  const v3 g = sample_adjoint(&s, filter, adj_density);
  sampler_flush(&s, filter);
  adj_pos[0] = g.x; adj_pos[1] = g.y; adj_pos[2] = g.z;
  return 0;
}

/* the ray (start, direction) of every pixel as the march computes it, B H W 3 each */
int oracle_camera_rays(const OracleInputs* in, OracleTensor* start, OracleTensor* dir) {
  if (in->camera_mode < 0 || in->camera_mode > 2) return 2;
  for (int b = 0; b < in->batch; ++b)
    for (int y = 0; y < in->height; ++y)
      for (int x = 0; x < in->width; ++x) {
        v3 s, d;
        compute_ray(in, x, y, b, &s, &d);
        *at4(start, b, y, x, 0) = s.x; *at4(start, b, y, x, 1) = s.y; *at4(start, b, y, x, 2) = s.z;
        *at4(dir, b, y, x, 0) = d.x; *at4(dir, b, y, x, 1) = d.y; *at4(dir, b, y, x, 2) = d.z;
      }
  return 0;
}

/* n positions volumePos(t_k), t_k = tmin + k*step, of one ray, and their adjoint */
int oracle_ray_steps(const real_t* start, const real_t* dir, const real_t* box_min, const real_t* voxel, real_t tmin,
                     real_t step, int n, real_t* pos) {
  RaySetup r;
  r.start = mk3(start[0], start[1], start[2]); r.dir = mk3(dir[0], dir[1], dir[2]);
  r.bmin = mk3(box_min[0], box_min[1], box_min[2]); r.voxel = mk3(voxel[0], voxel[1], voxel[2]);
  r.step = step; r.tmin = tmin; r.tmax = tmin + n * step;
  for (int k = 0; k < n; ++k) {
    const v3 p = volume_pos(&r, r.tmin + k * r.step);
    pos[3 * k] = p.x; pos[3 * k + 1] = p.y; pos[3 * k + 2] = p.z;
  }
  return 0;
}

int oracle_ray_steps_adjoint(const real_t* start, const real_t* dir, const real_t* box_min, const real_t* voxel,
                             real_t tmin, real_t step, int n, const real_t* adj_pos, real_t* adj_start, real_t* adj_dir,
                             real_t* adj_step) {
  RaySetup r;
  r.start = mk3(start[0], start[1], start[2]); r.dir = mk3(dir[0], dir[1], dir[2]);
  r.bmin = mk3(box_min[0], box_min[1], box_min[2]); r.voxel = mk3(voxel[0], voxel[1], voxel[2]);
  r.step = step; r.tmin = tmin; r.tmax = tmin + n * step;
  v3 as = mk3(0, 0, 0), ad = mk3(0, 0, 0);
  real_t at = 0;
  for (int k = n - 1; k >= 0; --k)
    ray_step_adjoint(&r, r.tmin + k * r.step, k, mk3(adj_pos[3 * k], adj_pos[3 * k + 1], adj_pos[3 * k + 2]), &as, &ad,
                     &at);
  adj_start[0] = as.x; adj_start[1] = as.y; adj_start[2] = as.z;
  adj_dir[0] = ad.x; adj_dir[1] = ad.y; adj_dir[2] = ad.z;
  *adj_step = at;
  return 0;
}
