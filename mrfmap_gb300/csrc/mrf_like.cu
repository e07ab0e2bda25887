// mrf_like.cu -- per-view log-likelihood of a depth image under the belief
// field (src/cuda/gvdbkernels.cu:183-293, 1246-1274), with the frame sum
// (src/cuda/gvdbhelper.cu:10-14) fused as a deterministic two-level
// reduction: FP64 block partials, then one ordered pass over the partials.
#include "mrf_geometry.cuh"
#include "mrf_internal.h"

namespace mrf {

namespace {

constexpr int kLikeThreads = 128;

__device__ __forceinline__ double block_sum(double v) {
  __shared__ double sh[kLikeThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
  int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0) {
    for (int i = 0; i < kLikeThreads / 32; ++i) t += sh[i];
  }
  return t;
}

// One thread per pixel.  Visibility V = exp(-sum alpha l) with
// alpha = -ln(1 - p); each voxel adds (V_prev - V) * P(z | first return in
// the voxel); the tail adds V_end * P(z | no return).  No early stop: every
// active brick to the volume exit is visited.
__global__ void __launch_bounds__(kLikeThreads)
    k_likelihood(Geom g, Pose P, const float* __restrict__ depth, const float* __restrict__ belief,
                 float* __restrict__ out_img, double* __restrict__ partials) {
  int pix = blockIdx.x * blockDim.x + threadIdx.x;
  float val = 0.0f;
  if (pix < g.rows * g.cols) {
    float d = depth[pix];
    if (d > 0.0f) {
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
      val = logf(sum);
    }
    if (out_img) out_img[pix] = val;
  }
  double t = block_sum((double)val);
  if (threadIdx.x == 0) partials[blockIdx.x] = t;
}

__global__ void k_reduce_partials(const double* __restrict__ partials, int n, float* out) {
  __shared__ double sh[256];
  double v = 0.0;
  // fixed assignment of partials to threads and a fixed tree: reproducible
  for (int i = threadIdx.x; i < n; i += blockDim.x) v += partials[i];
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = (float)sh[0];
}

}  // namespace

int likelihood_blocks(const Geom& g) {
  return (g.rows * g.cols + kLikeThreads - 1) / kLikeThreads;
}

cudaError_t launch_likelihood(const Geom& g, const Pose& P, const float* depth, const float* belief,
                              float* out_img, double* partials, int nblocks, cudaStream_t s) {
  k_likelihood<<<nblocks, kLikeThreads, 0, s>>>(g, P, depth, belief, out_img, partials);
  return cudaGetLastError();
}

cudaError_t launch_reduce_partials(const double* partials, int n, float* out_sum, cudaStream_t s) {
  k_reduce_partials<<<1, 256, 0, s>>>(partials, n, out_sum);
  return cudaGetLastError();
}

}  // namespace mrf
