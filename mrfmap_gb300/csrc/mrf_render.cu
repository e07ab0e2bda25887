// mrf_render.cu -- evaluation renders over the belief field, on the same
// traversal as the likelihood (every active brick to the volume exit):
//   mode 0  expected depth            gvdbkernels.cu:295-354, 1332-1363
//   mode 1  accuracy (peak of the first-return density within 1 sigma)
//                                      gvdbkernels.cu:183-293, 1066-1104
//   mode 2  simple accuracy (first voxel above a threshold)
//                                      gvdbkernels.cu:135-181, 1106-1134
//   mode 3  occupancy at the first voxel past the measurement
//                                      gvdbkernels.cu:183-293, 1136-1162
// Labels of modes 1-3 are histogrammed (-1, 0, 1, 2) for the frame scores of
// src/cuda/gvdbhelper.cu:16-62 (integer counts: order-independent).
#include "mrf_geometry.cuh"
#include "mrf_internal.h"

namespace mrf {

namespace {

constexpr int kRenderThreads = 128;

template <int kMode>
__device__ float render_pixel(const Geom& g, const Pose& P, const float* __restrict__ belief, int pix,
                              float d, float thresh) {
  int x = pix % g.cols, y = pix / g.cols;
  const float* sg = lut_at(g, g.sigma, x, y);
  const float* bs = lut_at(g, g.bias, x, y);
  const int n = g.lookup_n;
  Ray ray;
  ray_setup(g, P, x, y, ray);
  float A = 0.0f, Vprev = 1.0f, sum = 0.0f, peak = 0.0f, s_last = 0.0f;
  int peak_ok = 0, occ = -1;
  bool run_open = false;
  Dda r;
  if (dda_init(r, g, ray)) {
    int64_t cur = -1;
    int slot = -1;
    int vx, vy, vz;
    float l, tin, te;
    while (dda_next(r, g, vx, vy, vz, l, tin, te)) {
      int64_t lin = brick_lin(g, vx, vy, vz);
      if (lin != cur) {
        // simple accuracy: a brick that ends past the return is a miss
        if (kMode == 2 && run_open && s_last >= d) return 0.0f;
        run_open = false;
        cur = lin;
        slot = g.brick_slot[lin];
      }
      if (slot < 0) continue;
      run_open = true;
      float p = belief[(int64_t)slot * kBrickVox + voxel_local(vx, vy, vz)];
      float s = fm(te, ray.mult);
      s_last = s;
      if (kMode == 2) {
        if (p >= thresh) return fabsf(s - d) <= g.res ? 1.0f : 2.0f;
        continue;
      }
      float dA = log1pf(-p) * l;
      A += dA;
      float V = expf(A);
      float dv = Vprev * -expm1f(dA);
      if (kMode == 0) {
        // z-depth of the voxel's corner (the GVDB atlas-to-world position)
        float zc = fabsf(P.m[2] * ((float)vx - ray.o[0]) + P.m[6] * ((float)vy - ray.o[1]) +
                         P.m[10] * ((float)vz - ray.o[2])) * g.res;
        sum += dv * zc;
      } else {
        float pd = fs(fa(s, poly_f(bs, n, s)), d);
        if (kMode == 1) {
          float w = dv / l;
          if (w > peak) {
            peak = w;
            peak_ok = fabsf(pd) <= poly_f(sg, n, s);
          }
        }
        if (kMode == 3 && pd > 0.0f && occ == -1) occ = p >= thresh ? 1 : 0;
      }
      Vprev = V;
    }
  }
  if (kMode == 0) return sum / (1.0f - Vprev + kFEps);
  if (kMode == 1) {
    if (peak > 0.0f && Vprev >= 0.9f) return fa(s_last, poly_f(bs, n, s_last)) <= d ? -1.0f : 0.0f;
    if (peak > 0.0f) return (float)peak_ok;
    return -1.0f;
  }
  if (kMode == 2) return (run_open && s_last >= d) ? 0.0f : -1.0f;
  return (float)occ;
}

template <int kMode>
__global__ void __launch_bounds__(kRenderThreads)
    k_render(Geom g, Pose P, const float* __restrict__ depth, const float* __restrict__ belief,
             float thresh, float* __restrict__ out, unsigned long long* __restrict__ counts) {
  __shared__ unsigned int hist[4];
  if (threadIdx.x < 4) hist[threadIdx.x] = 0;
  __syncthreads();
  int pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix < g.rows * g.cols) {
    float d = depth[pix];
    float v;
    if (kMode != 0 && !(d > 0.0f)) v = -1.0f;
    else v = render_pixel<kMode>(g, P, belief, pix, d, thresh);
    out[pix] = v;
    if (kMode != 0) {
      int k = (int)v + 1;
      if (k >= 0 && k < 4) atomicAdd(&hist[k], 1u);
    }
  }
  __syncthreads();
  if (kMode != 0 && threadIdx.x < 4 && hist[threadIdx.x])
    atomicAdd(&counts[threadIdx.x], (unsigned long long)hist[threadIdx.x]);
}

}  // namespace

cudaError_t launch_render(int mode, const Geom& g, const Pose& P, const float* depth,
                          const float* belief, float thresh, float* out, unsigned long long* counts,
                          cudaStream_t s) {
  int nb = (g.rows * g.cols + kRenderThreads - 1) / kRenderThreads;
  switch (mode) {
    case 0: k_render<0><<<nb, kRenderThreads, 0, s>>>(g, P, depth, belief, thresh, out, counts); break;
    case 1: k_render<1><<<nb, kRenderThreads, 0, s>>>(g, P, depth, belief, thresh, out, counts); break;
    case 2: k_render<2><<<nb, kRenderThreads, 0, s>>>(g, P, depth, belief, thresh, out, counts); break;
    case 3: k_render<3><<<nb, kRenderThreads, 0, s>>>(g, P, depth, belief, thresh, out, counts); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace mrf
