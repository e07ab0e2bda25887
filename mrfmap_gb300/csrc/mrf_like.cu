// mrf_like.cu -- per-view log-likelihood of a depth image under the belief
// field (src/cuda/gvdbkernels.cu:183-293, 1246-1274), with the frame sum
// (src/cuda/gvdbhelper.cu:10-14) fused as a deterministic two-level
// reduction: FP64 block partials, then one ordered pass over the partials.
#include "mrf_internal.h"
#include "mrf_like_pixel.cuh"

namespace mrf {

namespace {

constexpr int kLikeThreads = 128;

// One thread per pixel (per-pixel body in mrf_like_pixel.cuh).
__global__ void __launch_bounds__(kLikeThreads)
    k_likelihood(Geom g, Pose P, const float* __restrict__ depth, const float* __restrict__ belief,
                 float* __restrict__ out_img, double* __restrict__ partials) {
  int pix = blockIdx.x * blockDim.x + threadIdx.x;
  float val = 0.0f;
  if (pix < g.rows * g.cols) {
    float d = depth[pix];
    if (d > 0.0f) val = likelihood_pixel(g, P, belief, pix, d);
    if (out_img) out_img[pix] = val;
  }
  double t = like_block_sum<kLikeThreads>((double)val);
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
