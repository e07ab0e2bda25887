// mrf_warmnet.cu -- the learned warm start's network and its training
// kernels.  Three 3x3x3 convolutions over one 8^3 brick at a time
// (4 -> 16 -> 16 -> 1 channels, ReLU after the first two, zeros beyond the
// brick faces) predict a voxel's converged log-odds from four per-voxel
// features.  Every convolution -- forward, the input gradient (the same
// convolution with flipped, transposed weights) and the weight gradient --
// runs on the tensor cores as BF16 x BF16 -> FP32 (mma.sync m16n8k16) over
// operands staged in shared memory; FP32 master weights, Adam.  Weight and
// bias gradients are per-brick partials summed in brick order, so a
// training step is deterministic.
//
// Brick layout everywhere: voxel (x*8 + y)*8 + z, channels innermost.
#include <cuda_bf16.h>

#include <algorithm>

#include "mrf_internal.h"

namespace mrf {
namespace net {

constexpr int kThreads = 256;  // 8 warps; a warp owns four 16-voxel tiles
constexpr int kHaloVox = 1000;  // (8 + 2)^3
constexpr int kC0 = 4, kC1 = 16, kC2 = 16, kC3 = 1;
// parameter vector (fp32): W1[27][4][16] b1[16] W2[27][16][16] b2[16] W3[27][16][1] b3[1]
constexpr int oW1 = 0;
constexpr int oB1 = oW1 + 27 * kC0 * kC1;
constexpr int oW2 = oB1 + kC1;
constexpr int oB2 = oW2 + 27 * kC1 * kC2;
constexpr int oW3 = oB2 + kC2;
constexpr int oB3 = oW3 + 27 * kC2 * kC3;
constexpr int kNParams = oB3 + kC3;

__host__ __device__ constexpr int round16(int x) { return (x + 15) / 16 * 16; }

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t ld32(const __nv_bfloat16* p) {
  return *reinterpret_cast<const uint32_t*>(p);
}

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 lo, __nv_bfloat16 hi) {
  return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

template <typename T>
__device__ __forceinline__ float to_f(T v);
template <>
__device__ __forceinline__ float to_f<float>(float v) { return v; }
template <>
__device__ __forceinline__ float to_f<__nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }

// halo position of voxel v's window origin; tap offsets inside the window
__device__ __forceinline__ int halo_base(int v) { return ((v >> 6) * 10 + ((v >> 3) & 7)) * 10 + (v & 7); }
__device__ __forceinline__ int tap_off(int tap) { return ((tap / 9) * 10 + (tap / 3) % 3) * 10 + tap % 3; }

// one brick's input with a one-voxel zero halo: sIn[h][CIN] (bf16)
template <int CIN, int CIN_G, typename TIn>
__device__ __forceinline__ void stage_input(__nv_bfloat16* sIn, const TIn* __restrict__ X, int64_t b) {
  const TIn* src = X + b * 512 * CIN_G;
  for (int i = threadIdx.x; i < kHaloVox * CIN; i += kThreads) {
    const int h = i / CIN, c = i % CIN;
    const int x = h / 100 - 1, y = (h / 10) % 10 - 1, z = h % 10 - 1;
    float v = 0.0f;
    if (c < CIN_G && x >= 0 && x < 8 && y >= 0 && y < 8 && z >= 0 && z < 8)
      v = to_f(src[((x * 8 + y) * 8 + z) * CIN_G + c]);
    sIn[i] = __float2bfloat16_rn(v);
  }
}

// Convolution as an implicit GEMM: rows = the brick's 512 voxels, columns =
// COUT output channels, reduction k = tap * CIN + c (padded to 16).  MODE 0:
// forward weights W[tap][c][n] of a layer with CIN_G inputs and COUT_G
// outputs.  MODE 1: input gradient of a layer whose forward weights are
// W[tap][n][c] (n < COUT_G its inputs, c < CIN_G its outputs), taps flipped.
// EPI 0: + bias, ReLU -> bf16 [512][COUT_G]; 1: + bias -> fp32 [512]
// (COUT_G == 1); 2: times (prev > 0), the ReLU derivative -> bf16.
template <int CIN, int CIN_G, int COUT, int COUT_G, int MODE, int EPI, typename TIn>
__global__ void __launch_bounds__(kThreads)
    k_conv(const TIn* __restrict__ X, const float* __restrict__ W, const float* __restrict__ bias,
           const __nv_bfloat16* __restrict__ prev, void* __restrict__ out) {
  constexpr int KP = round16(27 * CIN);
  constexpr int NT = COUT / 8;
  __shared__ __align__(16) __nv_bfloat16 sIn[kHaloVox * CIN];
  __shared__ __align__(16) __nv_bfloat16 sW[COUT * KP];
  const int64_t b = blockIdx.x;
  stage_input<CIN, CIN_G>(sIn, X, b);
  for (int i = threadIdx.x; i < COUT * KP; i += kThreads) {
    const int n = i / KP, k = i % KP;
    const int tap = k / CIN, c = k % CIN;
    float v = 0.0f;
    if (n < COUT_G && tap < 27 && c < CIN_G)
      v = MODE == 0 ? W[(tap * CIN_G + c) * COUT_G + n] : W[((26 - tap) * COUT_G + n) * CIN_G + c];
    sW[i] = __float2bfloat16_rn(v);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, t = lane & 3;
  int hb[4][2];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int v0 = (warp * 4 + i) * 16 + g;
    hb[i][0] = halo_base(v0);
    hb[i][1] = halo_base(v0 + 8);
  }
  float acc[4][NT][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < NT; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.0f;
  for (int ks = 0; ks < KP / 16; ++ks) {
    const int kA = ks * 16 + 2 * t, kB = kA + 8;
    const int tapA = kA / CIN, cA = kA % CIN, tapB = kB / CIN, cB = kB % CIN;
    const bool okA = tapA < 27, okB = tapB < 27;
    const int offA = okA ? tap_off(tapA) : 0, offB = okB ? tap_off(tapB) : 0;
    uint32_t bw[NT][2];
#pragma unroll
    for (int j = 0; j < NT; ++j) {
      const int n = j * 8 + g;
      bw[j][0] = ld32(sW + n * KP + kA);
      bw[j][1] = ld32(sW + n * KP + kB);
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      uint32_t a[4];
      a[0] = okA ? ld32(sIn + (hb[i][0] + offA) * CIN + cA) : 0u;
      a[1] = okA ? ld32(sIn + (hb[i][1] + offA) * CIN + cA) : 0u;
      a[2] = okB ? ld32(sIn + (hb[i][0] + offB) * CIN + cB) : 0u;
      a[3] = okB ? ld32(sIn + (hb[i][1] + offB) * CIN + cB) : 0u;
#pragma unroll
      for (int j = 0; j < NT; ++j) mma_bf16(acc[i][j], a, bw[j][0], bw[j][1]);
    }
  }
  // epilogue: rows g and g + 8 of each tile, columns j*8 + 2t, +1
#pragma unroll
  for (int i = 0; i < 4; ++i) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int v = (warp * 4 + i) * 16 + g + 8 * h;
      const int64_t row = b * 512 + v;
#pragma unroll
      for (int j = 0; j < NT; ++j) {
        const int n = j * 8 + 2 * t;
        float y0 = acc[i][j][2 * h], y1 = acc[i][j][2 * h + 1];
        if (EPI == 1) {
          if (n == 0) static_cast<float*>(out)[row] = y0 + bias[0];
          continue;
        }
        if (n >= COUT_G) continue;
        if (EPI == 0) {
          y0 = fmaxf(y0 + bias[n], 0.0f);
          y1 = fmaxf(y1 + bias[n + 1], 0.0f);
        } else {
          const __nv_bfloat16* pv = prev + row * COUT_G + n;
          if (!(__bfloat162float(pv[0]) > 0.0f)) y0 = 0.0f;
          if (!(__bfloat162float(pv[1]) > 0.0f)) y1 = 0.0f;
        }
        *reinterpret_cast<uint32_t*>(static_cast<__nv_bfloat16*>(out) + row * COUT_G + n) =
            pack2(__float2bfloat16_rn(y0), __float2bfloat16_rn(y1));
      }
    }
  }
}

// Weight gradient of one brick: D[k][n] = sum_v Xwin[v][k] * dZ[v][n], an
// implicit GEMM with rows k (tap * CIN + c, padded to 16), columns n and the
// brick's 512 voxels as the reduction; written in the weight layout
// [tap][c][n] to part[b], with the bias gradient sum_v dZ[v][n] to pbias[b].
template <int CIN, int CIN_G, int COUT, int COUT_G, typename TIn, typename TDz>
__global__ void __launch_bounds__(kThreads)
    k_conv_wgrad(const TIn* __restrict__ X, const TDz* __restrict__ dZ, float* __restrict__ part,
                 float* __restrict__ pbias) {
  constexpr int KP = round16(27 * CIN);
  constexpr int MT = KP / 16;
  constexpr int NT = COUT / 8;
  constexpr int MPW = (MT + 7) / 8;  // row tiles per warp
  __shared__ __align__(16) __nv_bfloat16 sIn[kHaloVox * CIN];
  __shared__ __align__(16) __nv_bfloat16 sDz[COUT * 512];
  const int64_t b = blockIdx.x;
  stage_input<CIN, CIN_G>(sIn, X, b);
  for (int i = threadIdx.x; i < COUT * 512; i += kThreads) {
    const int n = i / 512, v = i % 512;
    sDz[i] = __float2bfloat16_rn(n < COUT_G ? to_f(dZ[(b * 512 + v) * COUT_G + n]) : 0.0f);
  }
  __syncthreads();
  if (threadIdx.x < COUT_G) {
    // bias gradient from the same bf16 operands, summed in voxel order
    float s = 0.0f;
    for (int v = 0; v < 512; ++v) s += __bfloat162float(sDz[threadIdx.x * 512 + v]);
    pbias[b * COUT_G + threadIdx.x] = s;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, t = lane & 3;
  float acc[MPW][NT][4];
#pragma unroll
  for (int i = 0; i < MPW; ++i)
#pragma unroll
    for (int j = 0; j < NT; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.0f;
  // row k of tile m: tap and channel of rows g and g + 8
  int offr[MPW][2], cr[MPW][2];
  bool okr[MPW][2];
#pragma unroll
  for (int i = 0; i < MPW; ++i)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int mt = warp + 8 * i;
      const int k = mt * 16 + g + 8 * h;
      const int tap = k / CIN;
      okr[i][h] = mt < MT && tap < 27;
      offr[i][h] = okr[i][h] ? tap_off(tap) : 0;
      cr[i][h] = k % CIN;
    }
  for (int ks = 0; ks < 32; ++ks) {
    const int v0 = ks * 16 + 2 * t;  // columns v0, v0+1 and v0+8, v0+9
    uint32_t bw[NT][2];
#pragma unroll
    for (int j = 0; j < NT; ++j) {
      const int n = j * 8 + g;
      bw[j][0] = ld32(sDz + n * 512 + v0);
      bw[j][1] = ld32(sDz + n * 512 + v0 + 8);
    }
    const int hv[4] = {halo_base(v0), halo_base(v0 + 1), halo_base(v0 + 8), halo_base(v0 + 9)};
#pragma unroll
    for (int i = 0; i < MPW; ++i) {
      if (warp + 8 * i >= MT) continue;
      uint32_t a[4];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        if (okr[i][h]) {
          const __nv_bfloat16* base = sIn + offr[i][h] * CIN + cr[i][h];
          a[h] = pack2(base[hv[0] * CIN], base[hv[1] * CIN]);
          a[h + 2] = pack2(base[hv[2] * CIN], base[hv[3] * CIN]);
        } else {
          a[h] = 0u;
          a[h + 2] = 0u;
        }
      }
#pragma unroll
      for (int j = 0; j < NT; ++j) mma_bf16(acc[i][j], a, bw[j][0], bw[j][1]);
    }
  }
  float* dst = part + b * (27 * CIN_G * COUT_G);
#pragma unroll
  for (int i = 0; i < MPW; ++i) {
    const int mt = warp + 8 * i;
    if (mt >= MT) continue;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int k = mt * 16 + g + 8 * h;
      const int tap = k / CIN, c = k % CIN;
      if (tap >= 27 || c >= CIN_G) continue;
#pragma unroll
      for (int j = 0; j < NT; ++j) {
        const int n = j * 8 + 2 * t;
        if (n < COUT_G) dst[(tap * CIN_G + c) * COUT_G + n] = acc[i][j][2 * h];
        if (n + 1 < COUT_G) dst[(tap * CIN_G + c) * COUT_G + n + 1] = acc[i][j][2 * h + 1];
      }
    }
  }
}

// grad[i] = sum over bricks (in brick order) of part[b][i]
__global__ void k_sum_parts(const float* __restrict__ part, int64_t nb, int n, float* __restrict__ grad) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float s = 0.0f;
  for (int64_t b = 0; b < nb; ++b) s += part[b * n + i];
  grad[i] = s;
}

// masked squared error on log-odds: dOut = 2 w (y - t) / norm; per-brick
// partial of sum w (y - t)^2
__global__ void __launch_bounds__(kThreads)
    k_loss(const float* __restrict__ y, const float* __restrict__ target, const float* __restrict__ w,
           float inv_norm, float* __restrict__ dy, float* __restrict__ lpart) {
  __shared__ float red[kThreads / 32];
  const int64_t b = blockIdx.x;
  float s = 0.0f;
  for (int v = threadIdx.x; v < 512; v += kThreads) {
    const int64_t i = b * 512 + v;
    const float e = y[i] - target[i];
    dy[i] = 2.0f * w[i] * e * inv_norm;
    s += w[i] * e * e;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float tot = 0.0f;
    for (int k = 0; k < kThreads / 32; ++k) tot += red[k];
    lpart[b] = tot;
  }
}

__global__ void k_sum_loss(const float* __restrict__ lpart, int64_t nb, float inv_norm,
                           float* __restrict__ loss) {
  if (blockIdx.x || threadIdx.x) return;
  double s = 0.0;
  for (int64_t b = 0; b < nb; ++b) s += lpart[b];
  *loss = (float)(s * inv_norm);
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m1,
                       float* __restrict__ m2, int n, float lr, float b1, float b2, float eps, float c1,
                       float c2) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float a = b1 * m1[i] + (1.0f - b1) * gi;
  const float v = b2 * m2[i] + (1.0f - b2) * gi * gi;
  m1[i] = a;
  m2[i] = v;
  p[i] -= lr * (a / c1) / (sqrtf(v / c2) + eps);
}

struct Work {
  __nv_bfloat16 *a1, *a2, *dz2, *dz1;
  float *y, *dy, *part, *pbias, *lpart;
};

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

inline size_t work_bytes(int64_t nb, Work* w, char* base) {
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char* p = base ? base + off : nullptr;
    off += align256(bytes);
    return p;
  };
  const size_t vox = (size_t)nb * 512;
  char* a1 = take(vox * kC1 * 2);
  char* a2 = take(vox * kC2 * 2);
  char* dz2 = take(vox * kC2 * 2);
  char* dz1 = take(vox * kC1 * 2);
  char* y = take(vox * 4);
  char* dy = take(vox * 4);
  char* part = take((size_t)nb * 27 * kC1 * kC2 * 4);
  char* pbias = take((size_t)nb * kC1 * 4);
  char* lpart = take((size_t)nb * 4);
  if (w) {
    w->a1 = reinterpret_cast<__nv_bfloat16*>(a1);
    w->a2 = reinterpret_cast<__nv_bfloat16*>(a2);
    w->dz2 = reinterpret_cast<__nv_bfloat16*>(dz2);
    w->dz1 = reinterpret_cast<__nv_bfloat16*>(dz1);
    w->y = reinterpret_cast<float*>(y);
    w->dy = reinterpret_cast<float*>(dy);
    w->part = reinterpret_cast<float*>(part);
    w->pbias = reinterpret_cast<float*>(pbias);
    w->lpart = reinterpret_cast<float*>(lpart);
  }
  return off;
}

cudaError_t forward(const float* P, const float* feat, int64_t nb, const Work& w, float* out,
                    cudaStream_t s) {
  const unsigned grid = (unsigned)nb;
  k_conv<4, 4, 16, 16, 0, 0, float><<<grid, kThreads, 0, s>>>(feat, P + oW1, P + oB1, nullptr, w.a1);
  k_conv<16, 16, 16, 16, 0, 0, __nv_bfloat16><<<grid, kThreads, 0, s>>>(w.a1, P + oW2, P + oB2, nullptr, w.a2);
  k_conv<16, 16, 8, 1, 0, 1, __nv_bfloat16><<<grid, kThreads, 0, s>>>(w.a2, P + oW3, P + oB3, nullptr, out);
  return cudaGetLastError();
}

cudaError_t gradients(const float* P, const float* feat, const float* target, const float* wt, int64_t nb,
                      float inv_norm, float* grad, float* loss, const Work& w, cudaStream_t s) {
  const unsigned grid = (unsigned)nb;
  cudaError_t e = forward(P, feat, nb, w, w.y, s);
  if (e != cudaSuccess) return e;
  k_loss<<<grid, kThreads, 0, s>>>(w.y, target, wt, inv_norm, w.dy, w.lpart);
  k_sum_loss<<<1, 32, 0, s>>>(w.lpart, nb, inv_norm, loss);
  // layer 3: dW3, db3; input gradient dZ2 = (dy * W3) masked by a2 > 0
  k_conv_wgrad<16, 16, 8, 1, __nv_bfloat16, float><<<grid, kThreads, 0, s>>>(w.a2, w.dy, w.part, w.pbias);
  k_sum_parts<<<(27 * kC2 + 255) / 256, 256, 0, s>>>(w.part, nb, 27 * kC2 * kC3, grad + oW3);
  k_sum_parts<<<1, 32, 0, s>>>(w.pbias, nb, kC3, grad + oB3);
  k_conv<2, 1, 16, 16, 1, 2, float><<<grid, kThreads, 0, s>>>(w.dy, P + oW3, nullptr, w.a2, w.dz2);
  // layer 2
  k_conv_wgrad<16, 16, 16, 16, __nv_bfloat16, __nv_bfloat16><<<grid, kThreads, 0, s>>>(w.a1, w.dz2, w.part,
                                                                                      w.pbias);
  k_sum_parts<<<(27 * kC1 * kC2 + 255) / 256, 256, 0, s>>>(w.part, nb, 27 * kC1 * kC2, grad + oW2);
  k_sum_parts<<<1, 32, 0, s>>>(w.pbias, nb, kC2, grad + oB2);
  k_conv<16, 16, 16, 16, 1, 2, __nv_bfloat16><<<grid, kThreads, 0, s>>>(w.dz2, P + oW2, nullptr, w.a1, w.dz1);
  // layer 1
  k_conv_wgrad<4, 4, 16, 16, float, __nv_bfloat16><<<grid, kThreads, 0, s>>>(feat, w.dz1, w.part, w.pbias);
  k_sum_parts<<<(27 * kC0 * kC1 + 255) / 256, 256, 0, s>>>(w.part, nb, 27 * kC0 * kC1, grad + oW1);
  k_sum_parts<<<1, 32, 0, s>>>(w.pbias, nb, kC1, grad + oB1);
  return cudaGetLastError();
}

}  // namespace net
}  // namespace mrf

using namespace mrf;

extern "C" {

int64_t mrf_net_num_params(void) { return net::kNParams; }

int64_t mrf_net_workspace_bytes(int64_t n_bricks) {
  if (n_bricks < 0) return -1;
  return (int64_t)net::work_bytes(n_bricks, nullptr, nullptr);
}

static mrf_status net_status(cudaError_t e) {
  if (e == cudaSuccess) return MRF_OK;
  mrf_internal_set_error(std::string("CUDA: ") + cudaGetErrorString(e));
  return MRF_ERR_CUDA;
}

static bool net_args_ok(const void* a, const void* b, const void* ws, int64_t nb) {
  if (!a || !b || !ws || nb < 1 || nb > 0x7FFFFFFF) {
    mrf_internal_set_error("invalid network arguments");
    return false;
  }
  return true;
}

mrf_status mrf_net_forward(const float* params, const float* feat, int64_t n_bricks, float* out,
                           void* workspace, void* stream) {
  if (!net_args_ok(params, feat, workspace, n_bricks) || !out) return MRF_ERR_INVALID;
  net::Work w;
  net::work_bytes(n_bricks, &w, static_cast<char*>(workspace));
  return net_status(net::forward(params, feat, n_bricks, w, out, static_cast<cudaStream_t>(stream)));
}

mrf_status mrf_net_gradients(const float* params, const float* feat, const float* target,
                             const float* weight, int64_t n_bricks, float norm, float* grads,
                             float* loss, void* workspace, void* stream) {
  if (!net_args_ok(params, feat, workspace, n_bricks) || !target || !weight || !grads || !loss ||
      !(norm > 0.0f))
    return MRF_ERR_INVALID;
  net::Work w;
  net::work_bytes(n_bricks, &w, static_cast<char*>(workspace));
  return net_status(net::gradients(params, feat, target, weight, n_bricks, 1.0f / norm, grads, loss, w,
                                   static_cast<cudaStream_t>(stream)));
}

mrf_status mrf_net_adam(float* params, const float* grads, float* m1, float* m2, int64_t n, float lr,
                        float beta1, float beta2, float eps, int step, void* stream) {
  if (!params || !grads || !m1 || !m2 || n < 1 || n > 0x7FFFFFFF || step < 1) {
    mrf_internal_set_error("invalid Adam arguments");
    return MRF_ERR_INVALID;
  }
  const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
  net::k_adam<<<(unsigned)((n + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      params, grads, m1, m2, (int)n, lr, beta1, beta2, eps, c1, c2);
  return net_status(cudaGetLastError());
}

}  // extern "C"
