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

// Per-voxel record of one pixel's ray (src/cuda/gvdbkernels.cu:573-672,
// 1365-1384): ten floats per active voxel along the ray to the volume exit
// -- [0] exit distance s, [1] belief, [2..3] voxel id (u64: slot*512 +
// local), [4] w = (V_prev - V) / l, [5] visibility V, [6..7] brick slot
// (u64), [8] brick-local x, y, z as bytes -- and the record count in the
// last float.  One thread: this is a debugging probe.
__global__ void k_pixel_diag(Geom g, Pose P, const float* __restrict__ belief, int x, int y,
                             float* __restrict__ out, int64_t n_floats) {
  if (blockIdx.x || threadIdx.x) return;
  constexpr int kStride = 10;
  const int64_t cap = (n_floats - 1) / kStride;
  Ray ray;
  ray_setup(g, P, x, y, ray);
  int64_t count = 0;
  float A = 0.0f, Vprev = 1.0f;
  Dda r;
  if (dda_init(r, g, ray)) {
    int64_t cur = -1;
    int slot = -1;
    int vx, vy, vz;
    float l, tin, te;
    while (dda_next(r, g, vx, vy, vz, l, tin, te)) {
      int64_t lin = brick_lin(g, vx, vy, vz);
      if (lin != cur) {
        cur = lin;
        slot = g.brick_slot[lin];
      }
      if (slot < 0) continue;
      if (count >= cap) break;
      const int loc = voxel_local(vx, vy, vz);
      const float p = belief[(int64_t)slot * kBrickVox + loc];
      A += log1pf(-p) * l;
      const float V = expf(A);
      float* rec = out + count * kStride;
      rec[0] = fm(te, ray.mult);
      rec[1] = p;
      reinterpret_cast<unsigned long long*>(out)[count * (kStride / 2) + 1] =
          (unsigned long long)slot * kBrickVox + loc;
      rec[4] = (Vprev - V) / l;
      rec[5] = V;
      reinterpret_cast<unsigned long long*>(out)[count * (kStride / 2) + 3] = (unsigned long long)slot;
      unsigned char* b = reinterpret_cast<unsigned char*>(rec + 8);
      b[0] = (unsigned char)(vx & 7);
      b[1] = (unsigned char)(vy & 7);
      b[2] = (unsigned char)(vz & 7);
      Vprev = V;
      ++count;
    }
  }
  out[n_floats - 1] = (float)count;
}

}  // namespace

cudaError_t launch_pixel_diag(const Geom& g, const Pose& P, const float* belief, int x, int y, float* out,
                              int64_t n_floats, cudaStream_t s) {
  k_pixel_diag<<<1, 1, 0, s>>>(g, P, belief, x, y, out, n_floats);
  return cudaGetLastError();
}

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
