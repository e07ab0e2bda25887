// mrf_like_pixel.cuh -- per-pixel log-likelihood of a depth return under the
// belief field (src/cuda/gvdbkernels.cu:183-293, 1246-1274).  Visibility
// V = exp(-sum alpha l) with alpha = -ln(1 - p); each voxel adds
// (V_prev - V) * P(z | first return in the voxel); the tail adds
// V_end * P(z | no return).  No early stop: every active brick to the volume
// exit is visited.
#pragma once
#include "mrf_geometry.cuh"
#include "mrf_internal.h"

namespace mrf {

__device__ __forceinline__ float likelihood_pixel(const Geom& g, const Pose& P,
                                                  const float* __restrict__ belief, int pix, float d) {
  int x = pix % g.cols, y = pix / g.cols;
  const float* sg = lut_at(g, g.sigma, x, y);
  const float* bs = lut_at(g, g.bias, x, y);
  const int n = g.lookup_n;
  Ray ray;
  ray_setup(g, P, x, y, ray);
  float A = 0.0f, Vprev = 1.0f, sum = 0.0f, prev_s = 0.0f, s_last = 0.0f;
  bool first_run = true, run_open = false;
  Dda r;
  if (dda_init(r, g, ray)) {
    int64_t cur = -1;
    int slot = -1;
    int vx, vy, vz;
    float l, tin, te;
    while (dda_next(r, g, vx, vy, vz, l, tin, te)) {
      int64_t lin = brick_lin(g, vx, vy, vz);
      if (lin != cur) {
        if (run_open) {
          run_open = false;
          // a brick hands s + bias(s) to the next as its previous s
          // (gvdbkernels.cu:209, 292)
          prev_s = s_last + poly_f(bs, n, s_last);
        }
        cur = lin;
        slot = g.brick_slot[lin];
      }
      if (slot < 0) continue;
      if (!run_open) {
        run_open = true;
        if (first_run) {
          prev_s = fm(tin, ray.mult);
          first_run = false;
        }
      }
      float p = belief[(int64_t)slot * kBrickVox + voxel_local(vx, vy, vz)];
      float alpha = -log1pf(-p);
      float dA = -alpha * l;
      A += dA;
      float V = expf(A);
      float w = Vprev * -expm1f(dA);
      float s = fm(te, ray.mult);
      float Pz;
      if (s < kZMin) {
        Pz = 0.0f;
      } else {
        float pd = fs(fa(s, poly_f(bs, n, s)), d);
        if (fabsf(pd) <= fm(3.0f, poly_f(sg, n, s)))
          Pz = (1.0f - kLikeEps) * 0.5f * (potential(sg, bs, n, s, d) + potential(sg, bs, n, prev_s, d));
        else
          Pz = kLikeEps;
      }
      sum += w * Pz;
      Vprev = V;
      prev_s = s;
      s_last = s;
    }
  }
  sum += Vprev * (d >= kZMax ? 1.0f - kLikeEps : kLikeEps);
  return logf(sum);
}

// FP64 sum over the block, returned on thread 0 (blockDim.x == kThreadsLike)
template <int kThreadsLike>
__device__ __forceinline__ double like_block_sum(double v) {
  __shared__ double sh[kThreadsLike / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
  int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0) {
    for (int i = 0; i < kThreadsLike / 32; ++i) t += sh[i];
  }
  return t;
}

}  // namespace mrf
