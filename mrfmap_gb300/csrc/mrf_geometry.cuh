// mrf_geometry.cuh -- device geometry shared by the traversal, activation and
// likelihood kernels: pixel rays, the voxel DDA over the brick grid, the
// sensor polynomials and the depth potential.
//
// Every geometric quantity is built from separately rounded fp32 operations
// (__fmul_rn/__fadd_rn/__fdiv_rn, which nvcc never contracts into FMAs), in
// one fixed order, so the incidence lists are reproducible bit for bit on any
// host that evaluates the same IEEE operations.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "mrf_internal.h"

namespace mrf {

__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fd(float a, float b) { return __fdiv_rn(a, b); }

// depth clean-up of pixel i of a rows x cols image (src/GVDBImage.cpp:32-40):
// a non-finite return becomes "no return" (-1), and 848x480 images lose a
// 24-pixel left/right and a 20-pixel top/bottom border
__device__ __forceinline__ float clean_depth_value(float d, int i, int rows, int cols) {
  float v = isfinite(d) ? d : -1.0f;
  if (rows == 480 && cols == 848) {
    int x = i % cols, y = i / cols;
    if (x < 24 || x >= cols - 24 || y < 20 || y >= rows - 20) v = -1.0f;
  }
  return v;
}

// sensor polynomial p0 + p1 z (+ p2 z^2): src/cuda/gvdbkernels.cu:46-55
__device__ __forceinline__ float poly_f(const float* c, int n, float z) {
  if (n == 3) return fa(fa(fm(fm(z, z), c[2]), fm(z, c[1])), c[0]);
  return fa(fm(z, c[1]), c[0]);
}

// per-20x20-tile coefficient rows; tiles indexed by the upward (GL) row as in
// gvdbkernels.cu:47 (the reference flips the image on upload)
// a camera of another resolution than the tables' maps its pixel into the
// tables' image (identity for the map's own camera)
__device__ __forceinline__ const float* lut_at(const Geom& g, const float* lut, int x, int y) {
  int ygl = g.rows - 1 - y;
  int xs = (int)(((int64_t)x * g.lut_cols) / g.cols);
  int ys = (int)(((int64_t)ygl * g.lut_rows) / g.rows);
  return lut + ((ys / kLookupPx) * g.n_tiles_u + (xs / kLookupPx)) * g.lookup_n;
}

// exact-zero test of the fp32 depth potential (gvdbkernels.cu:57-72; the
// reference's __expf flushes below 2^-126)
__device__ __forceinline__ bool potential_is_zero(const float* sg, const float* bs, int n, float s,
                                                  float d) {
  float sig3 = fm(3.0f, poly_f(sg, n, s));
  float diff = fabsf(fs(d, fa(s, poly_f(bs, n, s))));
  float x = fd(diff, sig3);
  float h = fm(0.5f, fm(x, x));
  return !(h <= kMuCutoff);
}

// Gaussian depth potential with sigma' = 3 sigma(s)
__device__ __forceinline__ float potential(const float* sg, const float* bs, int n, float s, float d) {
  float sig3 = 3.0f * poly_f(sg, n, s);
  float diff = fabsf(d - (s + poly_f(bs, n, s)));
  float x = diff / sig3;
  return 0.398942f / sig3 * expf(-0.5f * x * x);
}

// pixel-centre ray through the reference's symmetric GL frustum
// (src/GVDBCamera.cpp:7-32, gvdbkernels.cu:1178-1179), origin and direction
// in voxel units, and the ray-parameter -> z-depth factor (gvdbkernels.cu:837)
struct Ray {
  float o[3], d[3], mult;
};

__device__ __forceinline__ void ray_setup(const Geom& g, const Pose& P, int x, int y, Ray& r) {
  float W = (float)g.cols, H = (float)g.rows;
  float ndcx = fs(fm(2.0f, fd(fa((float)x, 0.5f), W)), 1.0f);
  float ndcy = fs(fm(2.0f, fd(fa((float)y, 0.5f), H)), 1.0f);
  float rx = fm(ndcx, fd(g.cx, g.fx));
  float ry = fm(ndcy, fd(g.cy, g.fy));
  float dw0 = fa(fa(fm(P.m[0], rx), fm(P.m[1], ry)), P.m[2]);
  float dw1 = fa(fa(fm(P.m[4], rx), fm(P.m[5], ry)), P.m[6]);
  float dw2 = fa(fa(fm(P.m[8], rx), fm(P.m[9], ry)), P.m[10]);
  float n = __fsqrt_rn(fa(fa(fm(dw0, dw0), fm(dw1, dw1)), fm(dw2, dw2)));
  r.d[0] = fd(dw0, n);
  r.d[1] = fd(dw1, n);
  r.d[2] = fd(dw2, n);
  r.o[0] = fa(fd(P.m[3], g.res), g.off[0]);
  r.o[1] = fa(fd(P.m[7], g.res), g.off[1]);
  r.o[2] = fa(fd(P.m[11], g.res), g.off[2]);
  r.mult = fm(g.res, fabsf(fa(fa(fm(P.m[2], r.d[0]), fm(P.m[6], r.d[1])), fm(P.m[10], r.d[2]))));
}

// Amanatides & Woo voxel DDA over the box [blo, bhi) of the brick grid (the
// whole grid [0, 8*NB) unless the view is confined to a scene box).  The
// next boundary time of an axis is recomputed from the integer boundary each
// step, (b - o) * (1/d), so no error accumulates along the ray.
struct Dda {
  float ox, oy, oz, ix, iy, iz;
  float tx, ty, tz, tprev;
  int vx, vy, vz, sx, sy, sz;
  int guard;
  bool alive;
};

__device__ __forceinline__ bool dda_axis(float o, float d, int lo, int hi, float& inv, float& tn, float& tf) {
  if (d > 0.0f || d < 0.0f) {
    inv = fd(1.0f, d);
    float tA = fm(fs((float)lo, o), inv);
    float tB = fm(fs((float)hi, o), inv);
    tn = fminf(tA, tB);
    tf = fmaxf(tA, tB);
    return true;
  }
  inv = 0.0f;
  if (o < (float)lo || o >= (float)hi) return false;
  tn = -INFINITY;
  tf = INFINITY;
  return true;
}

__device__ __forceinline__ int dda_start(float o, float t0, float d, int lo, int hi) {
  int v = (int)floorf(fa(o, fm(t0, d)));
  return v < lo ? lo : (v > hi - 1 ? hi - 1 : v);
}

__device__ __forceinline__ float dda_tnext(int v, int s, float o, float inv) {
  if (s > 0) return fm(fs((float)(v + 1), o), inv);
  if (s < 0) return fm(fs((float)v, o), inv);
  return INFINITY;
}

__device__ __forceinline__ bool dda_init(Dda& r, const Geom& g, const Ray& ray) {
  float tn0, tf0, tn1, tf1, tn2, tf2;
  if (!dda_axis(ray.o[0], ray.d[0], g.blo[0], g.bhi[0], r.ix, tn0, tf0)) return false;
  if (!dda_axis(ray.o[1], ray.d[1], g.blo[1], g.bhi[1], r.iy, tn1, tf1)) return false;
  if (!dda_axis(ray.o[2], ray.d[2], g.blo[2], g.bhi[2], r.iz, tn2, tf2)) return false;
  float t0 = fmaxf(fmaxf(fmaxf(0.0f, tn0), tn1), tn2);
  float t1 = fminf(fminf(fminf(INFINITY, tf0), tf1), tf2);
  if (!(t0 < t1)) return false;
  r.ox = ray.o[0]; r.oy = ray.o[1]; r.oz = ray.o[2];
  r.vx = dda_start(ray.o[0], t0, ray.d[0], g.blo[0], g.bhi[0]);
  r.vy = dda_start(ray.o[1], t0, ray.d[1], g.blo[1], g.bhi[1]);
  r.vz = dda_start(ray.o[2], t0, ray.d[2], g.blo[2], g.bhi[2]);
  r.sx = ray.d[0] > 0.0f ? 1 : (ray.d[0] < 0.0f ? -1 : 0);
  r.sy = ray.d[1] > 0.0f ? 1 : (ray.d[1] < 0.0f ? -1 : 0);
  r.sz = ray.d[2] > 0.0f ? 1 : (ray.d[2] < 0.0f ? -1 : 0);
  r.tx = dda_tnext(r.vx, r.sx, r.ox, r.ix);
  r.ty = dda_tnext(r.vy, r.sy, r.oy, r.iy);
  r.tz = dda_tnext(r.vz, r.sz, r.oz, r.iz);
  r.tprev = t0;
  r.alive = true;
  r.guard = 2 * ((g.bhi[0] - g.blo[0]) + (g.bhi[1] - g.blo[1]) + (g.bhi[2] - g.blo[2])) + 8;
  return true;
}

// emits the current voxel (vx,vy,vz), its segment length, entry and exit
// parameters, then steps to the next voxel; ties step x before y before z
__device__ __forceinline__ bool dda_next(Dda& r, const Geom& g, int& vx, int& vy, int& vz,
                                         float& len, float& tin, float& texit) {
  if (!r.alive || r.guard-- <= 0) return false;
  vx = r.vx; vy = r.vy; vz = r.vz;
  tin = r.tprev;
  float te;
  if (r.tx <= r.ty && r.tx <= r.tz) {
    te = r.tx;
    r.vx += r.sx;
    if (r.vx < g.blo[0] || r.vx >= g.bhi[0]) r.alive = false;
    else r.tx = dda_tnext(r.vx, r.sx, r.ox, r.ix);
  } else if (r.ty <= r.tz) {
    te = r.ty;
    r.vy += r.sy;
    if (r.vy < g.blo[1] || r.vy >= g.bhi[1]) r.alive = false;
    else r.ty = dda_tnext(r.vy, r.sy, r.oy, r.iy);
  } else {
    te = r.tz;
    r.vz += r.sz;
    if (r.vz < g.blo[2] || r.vz >= g.bhi[2]) r.alive = false;
    else r.tz = dda_tnext(r.vz, r.sz, r.oz, r.iz);
  }
  float l = fs(te, tin);
  len = l < 0.0f ? 0.0f : l;
  texit = te;
  r.tprev = fmaxf(r.tprev, te);
  return true;
}

__device__ __forceinline__ int64_t brick_lin(const Geom& g, int vx, int vy, int vz) {
  return ((int64_t)(vx >> 3) * g.NB[1] + (vy >> 3)) * g.NB[2] + (vz >> 3);
}

__device__ __forceinline__ uint32_t voxel_local(int vx, int vy, int vz) {
  return (uint32_t)((((vx & 7) << 3) | (vy & 7)) << 3 | (vz & 7));
}

}  // namespace mrf
