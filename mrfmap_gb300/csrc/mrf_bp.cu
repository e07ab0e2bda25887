// mrf_bp.cu -- the BP hot loop over the incidence lists.
//
//   k_pair_prepare : per (camera, voxel) pair, the cavity probability
//                    q = P(empty) excluding the camera's own message
//                    (src/cuda/gvdbkernels.cu:764-773)
//   k_ray_bp       : per ray, Pre pass (tau accumulation with the reference's
//                    per-brick visibility reset, gvdbkernels.cu:689-819), the
//                    infinity term (gvdbkernels.cu:1196-1208) and the Post pass
//                    (ray->voxel messages, gvdbkernels.cu:824-1038), all as
//                    warp-wide log-domain prefix scans
//   k_pair_update  : per pair, the length-weighted message average, new
//                    log-odds message, total log-odds and belief
//                    (gvdbkernels.cu:457-479); a segmented sum over the
//                    voxel-sorted incidence permutation -- no atomics, fixed
//                    summation order
#include <algorithm>

#include "mrf_internal.h"

namespace mrf {

namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;

__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }

template <typename T>
__device__ __forceinline__ T warp_incl_scan(T v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T u = __shfl_up_sync(kFull, v, o);
    if (lane >= o) v += u;
  }
  return v;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

__global__ void k_pair_prepare(const uint32_t* __restrict__ pair_vox, const float* __restrict__ m,
                               const float* __restrict__ L, float2* __restrict__ q, uint32_t p0,
                               uint32_t p1) {
  uint32_t p = p0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= p1) return;
  float eta = L[pair_vox[p]] - m[p];
  float qq = clampf(1.0f / (1.0f + expf(eta)), kFEps, 1.0f - kFEps);
  q[p] = make_float2(qq, logf(qq));
}

// Accumulator type for the tau sums: fp32 for short rays, FP64 for rays with
// more than kLongRay incidences (their sums run long enough for fp32
// cancellation in R = T - F - tau to matter).
template <typename Acc>
__device__ __forceinline__ void ray_bp_warp(const RayMeta& me, const uint32_t* __restrict__ inc_pair,
                                            const float* __restrict__ inc_len,
                                            const float* __restrict__ inc_mu,
                                            const float2* __restrict__ pq, float* __restrict__ inc_pl,
                                            int fix_reset, int lane) {
  const int n_pre = me.n_pre, n_post = me.n_post;
  const int r0 = fix_reset ? 0 : me.r0;
  const int rinf = fix_reset ? 0 : me.rinf;
  const uint32_t off = me.off;
  // ---- Pre: T = sum_i V_i (1 - q_i) mu_i, visibility from r0 -------------
  float carryA = 0.0f;
  Acc T = 0;
  for (int base = r0; base < n_pre; base += 32) {
    int i = base + lane;
    float a = 0.0f, w = 0.0f, mu = 0.0f, q = 1.0f;
    if (i < n_pre) {
      float2 qq = pq[inc_pair[off + i]];
      q = qq.x;
      a = inc_len[off + i] * qq.y;
      mu = inc_mu[off + i];
    }
    float A = carryA + warp_incl_scan(a, lane);
    if (mu != 0.0f) w = expf(A) * (1.0f - q) * mu;
    T += (Acc)warp_sum(w);
    carryA = __shfl_sync(kFull, A, 31);
  }
  // ---- infinity term: visibility at the end of Pre ------------------------
  if (me.flags & 1u) {
    float Ainf;
    if (rinf == r0) {
      Ainf = carryA;
    } else {
      float s = 0.0f;
      for (int i = rinf + lane; i < n_pre; i += 32) s += inc_len[off + i] * pq[inc_pair[off + i]].y;
      Ainf = warp_sum(s);
    }
    T += (Acc)expf(Ainf);
  }
  // ---- Post: messages p_i for i < n_post -----------------------------------
  carryA = 0.0f;
  Acc carryF = 0;
  for (int base = 0; base < n_post; base += 32) {
    int i = base + lane;
    bool valid = i < n_post;
    float a = 0.0f, len = 0.0f, mu = 0.0f, q = 1.0f;
    if (valid) {
      float2 qq = pq[inc_pair[off + i]];
      q = qq.x;
      len = inc_len[off + i];
      a = len * qq.y;
      mu = inc_mu[off + i];
    }
    float A = carryA + warp_incl_scan(a, lane);
    float V = expf(A);
    float tau = valid ? V * (1.0f - q) * mu : 0.0f;
    float tincl = warp_incl_scan(tau, lane);
    float texcl = tincl - tau;
    Acc F = carryF + (Acc)texcl;
    Acc R = T - F - (Acc)tau;
    float mu1 = (float)(F + (Acc)(V * mu));
    float mu0 = (float)(F + R / (Acc)q);
    float p = clampf(mu1 / (mu1 + mu0 + 1e-7f), kFEps, 1.0f - kFEps);
    if (valid) inc_pl[off + i] = p * len;
    carryA = __shfl_sync(kFull, A, 31);
    carryF += (Acc)__shfl_sync(kFull, tincl, 31);
  }
}

__global__ void __launch_bounds__(256) k_ray_bp(const RayMeta* __restrict__ meta, uint32_t r0,
                                                uint32_t r1, const uint32_t* __restrict__ inc_pair,
                                                const float* __restrict__ inc_len,
                                                const float* __restrict__ inc_mu,
                                                const float2* __restrict__ pq,
                                                float* __restrict__ inc_pl, int fix_reset) {
  const int lane = threadIdx.x & 31;
  const uint32_t wpb = blockDim.x >> 5;
  for (uint32_t r = r0 + blockIdx.x * wpb + (threadIdx.x >> 5); r < r1; r += gridDim.x * wpb) {
    RayMeta me = meta[r];
    if (me.n_pre == 0) continue;
    if (me.n_pre > kLongRay)
      ray_bp_warp<double>(me, inc_pair, inc_len, inc_mu, pq, inc_pl, fix_reset, lane);
    else
      ray_bp_warp<float>(me, inc_pair, inc_len, inc_mu, pq, inc_pl, fix_reset, lane);
  }
}

// Pair update.  The segment of a pair (its incidences in the voxel-grouped
// permutation) is summed by a group of kGroup lanes striding through it, so
// the permutation reads coalesce; the group's partial sums combine in a fixed
// xor tree (deterministic).  Pairs with more than kLongSeg incidences (voxels
// next to the camera, crossed by hundreds of rays) are skipped here and summed
// by a whole warp in k_pair_update_long, which keeps the groups balanced.
constexpr int kGroup = 8;
constexpr uint32_t kLongSeg = 64;

__device__ __forceinline__ void apply_pair(uint32_t p, float acc, float c, const uint32_t* pair_vox,
                                           float* m, float* L, float* belief, float* dm, int jacobi) {
  float a = clampf(acc / c, kFEps, 1.0f - kFEps);
  float mn = logf(a) - logf(1.0f - a);
  float mo = m[p];
  m[p] = mn;
  if (jacobi) {
    dm[p] = mn - mo;
    return;
  }
  uint32_t v = pair_vox[p];
  float Lv = L[v] + (mn - mo);
  L[v] = Lv;
  belief[v] = 1.0f - clampf(1.0f / (1.0f + expf(Lv)), kFEps, 1.0f - kFEps);
}

__global__ void __launch_bounds__(256) k_pair_update(const uint32_t* __restrict__ pair_vox,
                              float* __restrict__ m, const float* __restrict__ cum,
                              const uint32_t* __restrict__ seg, const uint32_t* __restrict__ perm,
                              const float* __restrict__ pl, float* __restrict__ L,
                              float* __restrict__ belief, float* __restrict__ dm, uint32_t p0,
                              uint32_t p1, int jacobi) {
  const int gl = threadIdx.x & (kGroup - 1);
  uint32_t p = p0 + (blockIdx.x * blockDim.x + threadIdx.x) / kGroup;
  bool active = p < p1;
  float c = 0.0f;
  uint32_t s = 0, e = 0;
  if (active) {
    c = cum[p];
    s = seg[p];
    e = seg[p + 1];
  }
  bool upd = active && c > kCumLenGate && (e - s) <= kLongSeg;
  float acc = 0.0f;
  if (upd)
    for (uint32_t k = s + gl; k < e; k += kGroup) acc += pl[perm[k]];
#pragma unroll
  for (int o = kGroup / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(kFull, acc, o);
  if (gl != 0 || !active) return;
  if (!(c > kCumLenGate)) {
    if (jacobi) dm[p] = __int_as_float(0x7fc00000);  // NaN: pair not updated
    return;
  }
  if (upd) apply_pair(p, acc, c, pair_vox, m, L, belief, dm, jacobi);
}

__global__ void __launch_bounds__(256) k_pair_update_long(const uint32_t* __restrict__ list,
                                   uint32_t n, const uint32_t* __restrict__ pair_vox,
                                   float* __restrict__ m, const float* __restrict__ cum,
                                   const uint32_t* __restrict__ seg,
                                   const uint32_t* __restrict__ perm, const float* __restrict__ pl,
                                   float* __restrict__ L, float* __restrict__ belief,
                                   float* __restrict__ dm, int jacobi) {
  const int lane = threadIdx.x & 31;
  for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < n;
       w += (gridDim.x * blockDim.x) >> 5) {
    uint32_t p = list[w];
    float c = cum[p];
    float acc = 0.0f;
    for (uint32_t k = seg[p] + lane; k < seg[p + 1]; k += 32) acc += pl[perm[k]];
    acc = warp_sum(acc);
    if (lane == 0 && c > kCumLenGate) apply_pair(p, acc, c, pair_vox, m, L, belief, dm, jacobi);
  }
}

// list of the pairs with long segments (built once per incidence build)
__global__ void k_long_flag(const uint32_t* __restrict__ seg, uint32_t p0, uint32_t p1,
                            uint32_t* __restrict__ flag) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t p = p0 + i;
  if (p < p1) flag[i] = (seg[p + 1] - seg[p]) > kLongSeg ? 1u : 0u;
}

__global__ void k_long_scatter(const uint32_t* __restrict__ flag, const uint32_t* __restrict__ scan,
                               uint32_t p0, uint32_t n, uint32_t* __restrict__ list) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && flag[i]) list[scan[i]] = p0 + i;
}

// Jacobi: total log-odds of each voxel moves by the sum of its cameras'
// message changes (pairs of a voxel grouped by a voxel-sorted CSR)
__global__ void k_voxel_apply(const uint32_t* __restrict__ vseg, const uint32_t* __restrict__ vpairs,
                              const uint32_t* __restrict__ vvox, uint32_t nvox,
                              const float* __restrict__ dm, float* __restrict__ L,
                              float* __restrict__ belief) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nvox) return;
  float s = 0.0f;
  bool any = false;
  for (uint32_t k = vseg[i]; k < vseg[i + 1]; ++k) {
    float d = dm[vpairs[k]];
    if (d == d) {  // pairs below the length gate carry NaN and are skipped
      s += d;
      any = true;
    }
  }
  if (!any) return;
  uint32_t v = vvox[i];
  float Lv = L[v] + s;
  L[v] = Lv;
  belief[v] = 1.0f - clampf(1.0f / (1.0f + expf(Lv)), kFEps, 1.0f - kFEps);
}

// moving a camera: take its messages out of the total log-odds
__global__ void k_remove_messages(const uint32_t* __restrict__ pair_vox, float* __restrict__ m,
                                  uint32_t p0, uint32_t p1, float* __restrict__ L,
                                  float* __restrict__ belief) {
  uint32_t p = p0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= p1) return;
  float mo = m[p];
  if (mo == 0.0f) return;
  uint32_t v = pair_vox[p];
  float Lv = L[v] - mo;
  L[v] = Lv;
  belief[v] = 1.0f - clampf(1.0f / (1.0f + expf(Lv)), kFEps, 1.0f - kFEps);
  m[p] = 0.0f;
}

__global__ void k_remap_scatter(const uint32_t* __restrict__ pv, const float* __restrict__ m,
                                uint32_t n, float* __restrict__ dense) {
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < n) dense[pv[p]] = m[p];
}

__global__ void k_remap_gather(const uint32_t* __restrict__ pv, float* __restrict__ m, uint32_t n,
                               const float* __restrict__ dense) {
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < n) m[p] = dense[pv[p]];
}

__global__ void k_fill(float* p, int64_t n, float v) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

__global__ void k_vflag(const uint32_t* __restrict__ sk, uint32_t n, uint32_t* __restrict__ flag) {
  uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) flag[k] = (k == 0 || sk[k] != sk[k - 1]) ? 1u : 0u;
}

__global__ void k_vassign(const uint32_t* __restrict__ sk, const uint32_t* __restrict__ flag,
                          const uint32_t* __restrict__ scan, uint32_t n, uint32_t* __restrict__ vvox,
                          uint32_t* __restrict__ vseg) {
  uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n || !flag[k]) return;
  vvox[scan[k]] = sk[k];
  vseg[scan[k]] = k;
}

__global__ void k_scatter_const(const uint32_t* __restrict__ idx, uint32_t n, float v,
                                float* __restrict__ dense) {
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < n) dense[idx[p]] = v;
}

inline unsigned blocks(int64_t n, int t) { return (unsigned)std::max<int64_t>(1, (n + t - 1) / t); }

}  // namespace

cudaError_t launch_pair_prepare(const BpArrays& a, uint32_t p0, uint32_t p1, cudaStream_t s) {
  if (p1 <= p0) return cudaSuccess;
  k_pair_prepare<<<blocks(p1 - p0, 256), 256, 0, s>>>(a.pair_vox, a.pair_m, a.L, a.pair_q, p0, p1);
  return cudaGetLastError();
}

cudaError_t launch_ray_bp(const BpArrays& a, uint32_t r0, uint32_t r1, int fix_reset, int num_sms,
                          cudaStream_t s) {
  if (r1 <= r0) return cudaSuccess;
  int64_t warps = r1 - r0;
  int64_t b = std::min<int64_t>(blocks(warps, 8), (int64_t)num_sms * 8);
  k_ray_bp<<<(unsigned)b, 256, 0, s>>>(a.meta, r0, r1, a.inc_pair, a.inc_len, a.inc_mu, a.pair_q,
                                       a.inc_pl, fix_reset);
  return cudaGetLastError();
}

cudaError_t launch_pair_update(const BpArrays& a, uint32_t p0, uint32_t p1, int jacobi,
                               cudaStream_t s) {
  if (p1 <= p0) return cudaSuccess;
  k_pair_update<<<blocks((int64_t)(p1 - p0) * kGroup, 256), 256, 0, s>>>(
      a.pair_vox, a.pair_m, a.pair_cum, a.pair_seg, a.perm, a.inc_pl, a.L, a.belief, a.pair_dm, p0,
      p1, jacobi);
  return cudaGetLastError();
}

cudaError_t launch_pair_update_long(const BpArrays& a, const uint32_t* list, uint32_t n, int jacobi,
                                    int num_sms, cudaStream_t s) {
  if (!n) return cudaSuccess;
  int64_t b = std::min<int64_t>(blocks((int64_t)n * 32, 256), (int64_t)num_sms * 8);
  k_pair_update_long<<<(unsigned)b, 256, 0, s>>>(list, n, a.pair_vox, a.pair_m, a.pair_cum,
                                                 a.pair_seg, a.perm, a.inc_pl, a.L, a.belief,
                                                 a.pair_dm, jacobi);
  return cudaGetLastError();
}

cudaError_t launch_long_flag(const uint32_t* seg, uint32_t p0, uint32_t p1, uint32_t* flag,
                             cudaStream_t s) {
  if (p1 <= p0) return cudaSuccess;
  k_long_flag<<<blocks(p1 - p0, 256), 256, 0, s>>>(seg, p0, p1, flag);
  return cudaGetLastError();
}

cudaError_t launch_long_scatter(const uint32_t* flag, const uint32_t* scan, uint32_t p0, uint32_t n,
                                uint32_t* list, cudaStream_t s) {
  if (!n) return cudaSuccess;
  k_long_scatter<<<blocks(n, 256), 256, 0, s>>>(flag, scan, p0, n, list);
  return cudaGetLastError();
}

cudaError_t launch_voxel_apply(const uint32_t* vseg, const uint32_t* vpairs, const uint32_t* vvox,
                               uint32_t nvox, const float* pair_dm, float* L, float* belief,
                               cudaStream_t s) {
  if (!nvox) return cudaSuccess;
  k_voxel_apply<<<blocks(nvox, 256), 256, 0, s>>>(vseg, vpairs, vvox, nvox, pair_dm, L, belief);
  return cudaGetLastError();
}

cudaError_t launch_remove_messages(const BpArrays& a, uint32_t p0, uint32_t p1, cudaStream_t s) {
  if (p1 <= p0) return cudaSuccess;
  k_remove_messages<<<blocks(p1 - p0, 256), 256, 0, s>>>(a.pair_vox, a.pair_m, p0, p1, a.L, a.belief);
  return cudaGetLastError();
}

cudaError_t launch_remap_scatter(const uint32_t* pair_vox, const float* pair_m, uint32_t n,
                                 float* dense, cudaStream_t s) {
  if (!n) return cudaSuccess;
  k_remap_scatter<<<blocks(n, 256), 256, 0, s>>>(pair_vox, pair_m, n, dense);
  return cudaGetLastError();
}

cudaError_t launch_remap_gather(const uint32_t* pair_vox, float* pair_m, uint32_t n,
                                const float* dense, cudaStream_t s) {
  if (!n) return cudaSuccess;
  k_remap_gather<<<blocks(n, 256), 256, 0, s>>>(pair_vox, pair_m, n, dense);
  return cudaGetLastError();
}

cudaError_t launch_fill_f32(float* p, int64_t n, float v, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_fill<<<blocks(n, 256), 256, 0, s>>>(p, n, v);
  return cudaGetLastError();
}

cudaError_t launch_vflag(const uint32_t* sk, uint32_t n, uint32_t* flag, cudaStream_t s) {
  if (!n) return cudaSuccess;
  k_vflag<<<blocks(n, 256), 256, 0, s>>>(sk, n, flag);
  return cudaGetLastError();
}

cudaError_t launch_vassign(const uint32_t* sk, const uint32_t* flag, const uint32_t* scan,
                           uint32_t n, uint32_t* vvox, uint32_t* vseg, cudaStream_t s) {
  if (!n) return cudaSuccess;
  k_vassign<<<blocks(n, 256), 256, 0, s>>>(sk, flag, scan, n, vvox, vseg);
  return cudaGetLastError();
}

cudaError_t launch_scatter_const(const uint32_t* idx, uint32_t n, float v, float* dense,
                                 cudaStream_t s) {
  if (!n) return cudaSuccess;
  k_scatter_const<<<blocks(n, 256), 256, 0, s>>>(idx, n, v, dense);
  return cudaGetLastError();
}

}  // namespace mrf
